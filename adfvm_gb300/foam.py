"""OpenFOAM case files and the solver status file, in the formats the reference reads and writes.

* Mesh: ``constant/polyMesh/{points, faces, owner, neighbour, boundary}``, binary (faces as a
  ``faceCompactList``: offsets then point labels) or ascii, as adFVM/mesh.py:177-279 reads
  (``Mesh.readFoam``, ``readFoamFile``, ``readFoamBoundary``) and mesh.py:345-407 writes them.
  A points or boundary file under ``<time>/polyMesh`` takes precedence over the constant one.
* Fields: ``<time>/<name>`` volScalarField / volVectorField with ``internalField`` and a
  ``boundaryField`` dict (field.py:198-264 reads, field.py:436-476 writes). Every entry that
  starts with ``uniform`` or ``nonuniform`` is returned as a float64 array (nFaces, dims) -
  ``value``, ``U0``, ``T0``, ``p0``, ``Tt``, ``pt``, ``direction`` - which is what
  ``BoundaryCondition.createInput`` makes of them (BCs.py:45-53 through mesh.extractField);
  every other entry stays a string, as the reference keeps it.
* Status: ``status.pkl`` = pickled ``[timeIndex, t, dt, result]`` (solver.py:185-205), or
  ``[checkpoint, result]`` for the adjoint sweep (apps/adjoint.py:154-158).

Binary payloads are skipped by their exact byte count, so payload bytes that happen to spell a
keyword or a bracket never confuse the parser.
"""
import os
import pickle
import re

import numpy as np

HEADER = (b'/*--------------------------------*- C++ -*----------------------------------*\\\n'
          b'| =========                 |                                                 |\n'
          b'| \\\\      /  F ield         | OpenFOAM: The Open Source CFD Toolbox           |\n'
          b'|  \\\\    /   O peration     | Version:  2.2.2                                 |\n'
          b'|   \\\\  /    A nd           | Web:      www.OpenFOAM.org                      |\n'
          b'|    \\\\/     M anipulation  |                                                 |\n'
          b'\\*---------------------------------------------------------------------------*/\n')
SEP = b'// * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * //\n'
# boundary types whose 'value' the writer replaces by the ghost-cell values (BCs.py:18-23)
VALUE_PATCHES = ('processor', 'processorCyclic', 'calculated', 'CBC_UPT', 'CBC_TOTAL_PT',
                 'nonReflectingOutletPressure', 'turbulentInletVelocity')
_NUM = rb'[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?'


class FoamFormatError(ValueError):
    pass


# ---------------------------------------------------------------- tokens

_WS = re.compile(rb'(?:\s+|//[^\n]*\n?|/\*.*?\*/)*', re.DOTALL)
_WORD = re.compile(rb'"[^"]*"|[A-Za-z0-9_.+\-<>:#$]+|[{}();\[\]]')
_SIZE = re.compile(rb'\s*(\d+)')


def _skip(buf, pos):
    return _WS.match(buf, pos).end()


def _token(buf, pos):
    pos = _skip(buf, pos)
    m = _WORD.match(buf, pos)
    if m is None:
        raise FoamFormatError('unexpected bytes at %d: %r' % (pos, buf[pos:pos + 20]))
    return m.group(0).decode(), m.end()


def _foamfile(buf):
    """(header dict, position after it)."""
    m = re.search(rb'FoamFile\s*\{', buf)
    if m is None:
        raise FoamFormatError('no FoamFile header')
    end = buf.index(b'}', m.end())
    d = {k.decode(): v.decode().strip().strip('"')
         for k, v in re.findall(rb'(\w+)[ \t]+([^;]+);', buf[m.end():end])}
    return d, end + 1


def _list_payload(buf, pos, n, dims, dtype, binary):
    """Parse '( ... )' holding n items of `dims` numbers, from pos (at or before the '(').
    Returns (array (n, dims), position after ')')."""
    pos = _skip(buf, pos)
    if buf[pos:pos + 1] != b'(':
        raise FoamFormatError('expected ( at %d' % pos)
    pos += 1
    if binary and n > 0:
        nb = n * dims * np.dtype(dtype).itemsize
        if len(buf) < pos + nb:
            raise FoamFormatError('binary list of %d items is truncated' % n)
        arr = np.frombuffer(buf[pos:pos + nb], dtype).reshape(n, dims).copy()
        pos = _skip(buf, pos + nb)
        if buf[pos:pos + 1] != b')':
            raise FoamFormatError('binary list of %d items does not end in )' % n)
        return arr, pos + 1
    depth, i = 1, pos
    while depth:
        c = buf[i:i + 1]
        if not c:
            raise FoamFormatError('unterminated list')
        depth += (c == b'(') - (c == b')')
        i += 1
    nums = re.findall(_NUM, buf[pos:i - 1])
    conv = float if np.dtype(dtype).kind == 'f' else int
    arr = np.array([conv(x) for x in nums], dtype)
    if arr.size != n * dims:
        raise FoamFormatError('list of %d x %d holds %d numbers' % (n, dims, arr.size))
    return arr.reshape(n, dims), i


def _entry(buf, pos, binary, nFaces):
    """An entry's value after its keyword, through its ';'. uniform/nonuniform values become
    float64 arrays (nFaces or the list's size, dims); anything else a stripped string."""
    start = _skip(buf, pos)
    word, after = _token(buf, start)
    if word == 'uniform':
        end = buf.index(b';', after)
        nums = [float(x) for x in re.findall(_NUM, buf[after:end])]
        return np.tile(np.array(nums, np.float64), (nFaces, 1)), end + 1
    if word == 'nonuniform':
        m = re.compile(rb'\s*List<(\w+)>\s*(\d+)').match(buf, after)
        if m is None:
            raise FoamFormatError('malformed nonuniform entry at %d' % after)
        kind, n = m.group(1).decode(), int(m.group(2))
        dims = {'scalar': 1, 'vector': 3}.get(kind)
        if dims is None:
            raise FoamFormatError('List<%s> is not supported' % kind)
        arr, pos = _list_payload(buf, m.end(), n, dims, np.float64, binary)
        pos = _skip(buf, pos)
        if buf[pos:pos + 1] != b';':
            raise FoamFormatError('expected ; after a list')
        return arr, pos + 1
    end = buf.index(b';', start)
    return buf[start:end].decode().strip(), end + 1


def _dict(buf, pos, binary, sizes):
    """'{ name { key entry; ... } ... }' from pos (at or before the '{'); sizes(name) is the
    patch's number of faces, for uniform entries. Returns (dict, position after '}')."""
    tok, pos = _token(buf, pos)
    if tok != '{':
        raise FoamFormatError('expected {')
    out = {}
    while True:
        name, pos = _token(buf, pos)
        if name == '}':
            return out, pos
        name = name.strip('"')
        tok, pos = _token(buf, pos)
        if tok != '{':
            raise FoamFormatError('expected { after %s' % name)
        entry = {}
        while True:
            key, pos = _token(buf, pos)
            if key == '}':
                break
            entry[key], pos = _entry(buf, pos, binary, sizes(name))
        if entry.get('type') == 'cyclicAMI':
            entry['type'] = 'cyclic'
        out[name] = entry


# ---------------------------------------------------------------- mesh

def _write_header(f, cls, obj, location=None):
    f.write(HEADER + b'FoamFile\n{\n')
    for k, v in (('version', '2.0'), ('format', 'binary'), ('class', cls), ('object', obj)):
        f.write(b'\t%s %s;\n' % (k.encode(), v.encode()))
    if location:
        f.write(b'\tlocation %s;\n' % location.encode())
    f.write(b'}\n' + SEP)


def write_mesh(case_dir, meshData):
    """constant/polyMesh of (points, faces, owner, neighbour, boundary), binary; faces are rows
    [nPoints, p0, ..] of equal length (the layout the geometry build takes)."""
    points, faces, owner, neighbour, boundary = meshData[:5]
    d = os.path.join(case_dir, 'constant', 'polyMesh')
    os.makedirs(d, exist_ok=True)
    faces = np.asarray(faces, np.int32)
    nF, k = faces.shape[0], faces.shape[1] - 1
    with open(os.path.join(d, 'points'), 'wb') as f:
        _write_header(f, 'vectorField', 'points', 'constant/polyMesh')
        f.write(b'\n%d\n(' % len(points) + np.ascontiguousarray(points, np.float64).tobytes() + b')\n\n' + SEP)
    with open(os.path.join(d, 'faces'), 'wb') as f:
        _write_header(f, 'faceCompactList', 'faces', 'constant/polyMesh')
        offsets = np.arange(0, nF * k + 1, k, dtype=np.int32)
        f.write(b'\n%d\n(' % len(offsets) + offsets.tobytes() + b')\n')
        f.write(b'%d\n(' % (nF * k) + np.ascontiguousarray(faces[:, 1:]).tobytes() + b')\n\n' + SEP)
    for name, arr in (('owner', owner), ('neighbour', neighbour)):
        with open(os.path.join(d, name), 'wb') as f:
            _write_header(f, 'labelList', name, 'constant/polyMesh')
            arr = np.ascontiguousarray(np.asarray(arr).reshape(-1), np.int32)
            f.write(b'\n%d\n(' % len(arr) + arr.tobytes() + b')\n\n' + SEP)
    write_boundary(os.path.join(d, 'boundary'), boundary)


def write_boundary(path, boundary):
    """polyBoundaryMesh in startFace order (mesh.py:385-407); derived keys are left out."""
    with open(path, 'wb') as f:
        _write_header(f, 'polyBoundaryMesh', 'boundary', 'constant/polyMesh')
        names = sorted(boundary, key=lambda x: (int(boundary[x]['startFace']), int(boundary[x]['nFaces'])))
        f.write(b'%d\n(\n' % len(names))
        for n in names:
            f.write(b'\t' + n.encode() + b'\n\t{\n')
            for key, v in boundary[n].items():
                if key.startswith('loc_') or key.startswith('_') or key == 'cellStartFace':
                    continue
                f.write(b'\t\t%s %s;\n' % (key.encode(), str(v).encode()))
            f.write(b'\t}\n')
        f.write(b')\n\n' + SEP)


def _faces_ascii(buf, pos, n):
    pos = _skip(buf, pos)
    if buf[pos:pos + 1] != b'(':
        raise FoamFormatError('expected ( before the faces')
    rows = re.compile(rb'\s*(\d+)\s*\(([^)]*)\)')
    out = []
    pos += 1
    for _ in range(n):
        m = rows.match(buf, pos)
        if m is None:
            raise FoamFormatError('malformed ascii face')
        out.append([int(m.group(1))] + [int(x) for x in m.group(2).split()])
        pos = m.end()
    if len({len(r) for r in out}) > 1:
        raise FoamFormatError('faces of different sizes are not supported')
    return np.array(out, np.int32).reshape(n, -1)


def read_list(path, dtype=None):
    """points (n, 3) float64, owner/neighbour (n,) int32, faces (n, 1 + k) int32 rows
    [k, p0 .. p(k-1)] (mesh.py:207-233); the class in the header picks the form."""
    buf = open(path, 'rb').read()
    hdr, pos = _foamfile(buf)
    binary = hdr.get('format', 'ascii') == 'binary'
    cls = hdr.get('class', '')
    m = _SIZE.match(buf, _skip(buf, pos))
    if m is None:
        raise FoamFormatError('%s: no list size' % path)
    n = int(m.group(1))
    if cls == 'faceCompactList':
        offsets, pos = _list_payload(buf, m.end(), n, 1, np.int32, binary)
        m2 = _SIZE.match(buf, pos)
        data, _ = _list_payload(buf, m2.end(), int(m2.group(1)), 1, np.int32, binary)
        offsets, data = offsets.reshape(-1), data.reshape(-1)
        counts = np.diff(offsets)
        if len(counts) and np.any(counts != counts[0]):
            raise FoamFormatError('faces of different sizes are not supported')
        k = int(counts[0]) if len(counts) else 4
        return np.hstack([np.full((len(counts), 1), k, np.int32), data.reshape(-1, k)]).astype(np.int32)
    if cls == 'faceList':
        if binary:
            raise FoamFormatError('binary faceList is not supported (write faceCompactList)')
        return _faces_ascii(buf, m.end(), n)
    if cls == 'vectorField':
        arr, _ = _list_payload(buf, m.end(), n, 3, dtype or np.float64, binary)
        return arr
    arr, _ = _list_payload(buf, m.end(), n, 1, dtype or np.int32, binary)
    return arr.reshape(-1)


def read_boundary(path):
    """polyBoundaryMesh -> {patch: {key: str, nFaces: int, startFace: int}} (mesh.py:254-279)."""
    buf = open(path, 'rb').read()
    hdr, pos = _foamfile(buf)
    binary = hdr.get('format') == 'binary'
    m = _SIZE.match(buf, _skip(buf, pos))
    n = int(m.group(1))
    tok, pos = _token(buf, m.end())
    if tok != '(':
        raise FoamFormatError('expected ( in the boundary file')
    boundary = {}
    for _ in range(n):
        name, pos = _token(buf, pos)
        tok, pos = _token(buf, pos)
        if tok != '{':
            raise FoamFormatError('expected { after patch %s' % name)
        p = {}
        while True:
            key, pos = _token(buf, pos)
            if key == '}':
                break
            p[key], pos = _entry(buf, pos, binary, 0)
        p['nFaces'] = int(p['nFaces'])
        p['startFace'] = int(p['startFace'])
        if p['type'] == 'cyclicAMI':
            p['type'] = 'cyclic'
        boundary[name.strip('"')] = p
    return boundary


def read_mesh(case_dir, time=None):
    """(points, faces, owner, neighbour, boundary) of a case (Mesh.readFoam)."""
    const = os.path.join(case_dir, 'constant', 'polyMesh')
    tdir = os.path.join(case_dir, time_name(time), 'polyMesh') if time is not None else None

    def pick(f):
        if tdir and os.path.exists(os.path.join(tdir, f)):
            return os.path.join(tdir, f)
        return os.path.join(const, f)
    points = read_list(pick('points'), np.float64)
    faces = read_list(os.path.join(const, 'faces'))
    owner = read_list(os.path.join(const, 'owner'), np.int32)
    neighbour = read_list(os.path.join(const, 'neighbour'), np.int32)
    return points, faces, owner, neighbour, read_boundary(pick('boundary'))


# ---------------------------------------------------------------- fields

def _write_list(f, key, arr, indent=b''):
    arr = np.ascontiguousarray(np.asarray(arr, np.float64).reshape(len(arr), -1))
    kind = b'vector' if arr.shape[1] == 3 else b'scalar'
    f.write(indent + key.encode() + b' nonuniform List<' + kind + b'>\n')
    f.write(b'%d\n(' % len(arr) + arr.tobytes() + b')\n;\n')


def _uniform(arr):
    """'uniform x' / 'uniform (x y z)' text of an array whose rows are all equal, else None;
    repr round-trips every float64 exactly."""
    arr = np.asarray(arr, np.float64).reshape(len(arr), -1)
    if len(arr) == 0 or not np.all(arr == arr[0]):
        return None
    v = [repr(float(x)) for x in arr[0]]
    return 'uniform ' + (v[0] if len(v) == 1 else '(' + ' '.join(v) + ')')


def write_field(time_dir, name, internal, boundary):
    """<time_dir>/<name>, binary (field.py:436-476): internal (nCells, 1|3); boundary
    {patch: {key: array | str}}. 'value' arrays are written as nonuniform binary lists, as the
    reference writes them; other arrays (U0, T0, p0, Tt, pt, direction) as 'uniform' text when
    all their rows are equal - the only form of those entries the reference's reader takes
    (it keeps them as text, field.py:247-253) - else as binary lists."""
    os.makedirs(time_dir, exist_ok=True)
    internal = np.asarray(internal, np.float64)
    internal = internal.reshape(len(internal), -1)
    with open(os.path.join(time_dir, name), 'wb') as f:
        _write_header(f, 'volVectorField' if internal.shape[1] == 3 else 'volScalarField', name)
        f.write(b'dimensions      [0 1 -1 0 0 0 0];\n')
        _write_list(f, 'internalField', internal)
        f.write(b'boundaryField\n{\n')
        for patch, b in boundary.items():
            f.write(b'\t' + patch.encode() + b'\n\t{\n')
            for key, v in b.items():
                if key.startswith('_'):
                    continue
                if isinstance(v, np.ndarray):
                    u = None if key == 'value' else _uniform(v)
                    if u is None:
                        _write_list(f, key, v, b'\t\t')
                    else:
                        f.write(b'\t\t%s %s;\n' % (key.encode(), u.encode()))
                else:
                    f.write(b'\t\t%s %s;\n' % (key.encode(), str(v).encode()))
            f.write(b'\t}\n')
        f.write(b'}\n')


def read_field(time_dir, name, mesh_boundary, nInternalCells):
    """(internal (nInternalCells, dims), boundary {patch: {key: array | str}})
    (IOField.readFoam, field.py:198-264)."""
    buf = open(os.path.join(time_dir, name), 'rb').read()
    hdr, pos = _foamfile(buf)
    binary = hdr.get('format', 'ascii') == 'binary'
    dims = 3 if hdr.get('class') == 'volVectorField' else 1
    m = re.compile(rb'internalField\b').search(buf, pos)
    if m is None:
        raise FoamFormatError('%s: no internalField' % name)
    internal, pos = _entry(buf, m.end(), binary, nInternalCells)
    if not isinstance(internal, np.ndarray) or internal.size != nInternalCells * dims:
        raise FoamFormatError('%s: internalField does not hold %d x %d values' % (name, nInternalCells, dims))
    internal = internal.reshape(nInternalCells, dims)
    m = re.compile(rb'boundaryField\b').search(buf, pos)
    if m is None:
        raise FoamFormatError('%s: no boundaryField' % name)

    def sizes(patch):
        return int(mesh_boundary[patch]['nFaces']) if patch in mesh_boundary else 0
    boundary, _ = _dict(buf, m.end(), binary, sizes)
    missing = [p for p in mesh_boundary if p not in boundary]
    if missing:
        raise FoamFormatError('%s: no boundary entry for %s' % (name, ', '.join(missing)))
    return internal, boundary


# ---------------------------------------------------------------- cases and status

def time_name(t):
    """Directory name of time t (Mesh.getTimeString, mesh.py:128-135)."""
    t = float(t)
    return '%d' % int(t) if t.is_integer() else '{0:.11f}'.format(t)


def times(case_dir):
    """Sorted times that have a directory (Mesh.getTimes, mesh.py:142-147)."""
    out = []
    for x in os.listdir(case_dir):
        try:
            out.append(float(x))
        except ValueError:
            pass
    return sorted(out)


def write_status(path, data):
    """status.pkl (Solver.writeStatusFile, solver.py:194-198)."""
    with open(path, 'wb') as f:
        pickle.dump(list(data), f)


def read_status(path):
    """status.pkl contents, or None when there is none (solver.py:185-192)."""
    if not os.path.exists(path):
        return None
    with open(path, 'rb') as f:
        return pickle.load(f)
