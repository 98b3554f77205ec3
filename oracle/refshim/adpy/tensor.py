"""NumPy stand-in for the adpy DSL that the reference's hot path is written in.

adpy (chaitan3/adpy, commit unknown) is an empty git submodule in the reference
(.gitmodules:1-3), so the reference cannot run as shipped. This module reconstructs the
semantics of the adpy API from its call sites in the reference (adFVM/density.py,
interp.py, riemann.py, op.py, timestep.py, BCs.py, solver.py, mesh.py) so that the
reference's OWN formula and driver code executes here, unmodified, on CPU in float64. No
adpy source is reproduced; the chosen semantics are:

* ``Variable``/``StaticVariable``/``StaticIntegerVariable``/``IntegerScalar`` are
  placeholders bound when a ``Function`` is called; ``Zeros(shape)`` is a zero array;
  ``v[start]`` (outside a kernel) is an offset view starting at row ``start`` of ``v``'s
  array, and ``v[a][b]`` is ``v[b]``.
* ``Kernel(f)(n, outputs)(*args)`` runs ``f`` once over element range ``[0, n)``:
  an argument used directly (or via ``index()``) is row ``offset+i`` of its array;
  ``x.extract(idx)`` gathers rows ``offset+idx`` of the full array; ``x.scalar()``
  broadcasts row 0. Results are written to the given outputs (copy-on-write, so every
  kernel call yields new arrays) or returned as new arrays.
* ``Tensor.collate(v0, i0, v1, i1, ...)`` scatter-adds into output rows; for element i the
  pairs are applied in argument order, elements in increasing i (the per-face loop of a
  generated CPU kernel). ``sum()`` accumulates sequentially in index order; ``reduce_max``
  is the maximum.
* ``x.stabilise(s)`` is ``x + s`` where ``x >= 0`` and ``x - s`` where ``x < 0``;
  ``Tensor.switch`` is a select; ``Tensor.max`` the elementwise maximum.
* Elementwise arithmetic is left-to-right IEEE double; dot/magSqr/tensordot/trace sum
  their products left to right.
* ``ExternalFunctionOp`` (MPI halo and allreduce ops) is the identity on one rank.
Test infrastructure only (fixture generation and oracle pinning).
"""
import numpy as np


class Container(object):
    pass


class _Info(object):
    def __init__(self):
        self.info = []


# ---------------------------------------------------------------- array-level graph

class Node(object):
    _counter = 0

    def __init__(self):
        Node._counter += 1
        self.uid = Node._counter
        self.args = [_Info()]

    def __getitem__(self, start):
        return OffsetView(self, start)

    def getReference(self):
        return self

    def __hash__(self):
        return self.uid

    def __eq__(self, other):
        return self is other


class Variable(Node):
    def __init__(self, shape=None, dtype=None):
        super().__init__()
        self.shape = shape
        self.dtype = dtype
        self.name = 'v%d' % self.uid

    def _eval(self, env):
        if self not in env.feed:
            raise KeyError('unbound placeholder %s %s' % (self.name, self.shape))
        val = env.feed[self]
        if isinstance(val, (int, np.integer)):
            return int(val)
        arr = np.asarray(val)
        if arr.ndim == 1:
            arr = arr.reshape(-1, 1)
        return (arr, 0)

    def _dummy(self):
        shape = [1] + [int(s) if isinstance(s, (int, np.integer)) else 1 for s in (self.shape or (1,))[1:]]
        if len(shape) == 1:
            shape.append(1)
        return (np.ones(shape), 0)


class StaticVariable(Variable):
    pass


class StaticIntegerVariable(Variable):
    def _dummy(self):
        shape = [1] + [int(s) if isinstance(s, (int, np.integer)) else 1 for s in (self.shape or (1,))[1:]]
        if len(shape) == 1:
            shape.append(1)
        return (np.zeros(shape, np.int64), 0)


class IntegerScalar(Variable):
    def __init__(self):
        super().__init__(())

    def _dummy(self):
        return 0


def _resolve_int(x, env):
    if isinstance(x, Node):
        return int(env.value(x))
    return int(x)


class Zeros(Node):
    def __init__(self, shape, dtype=None):
        super().__init__()
        self.shape = shape

    def _eval(self, env):
        shape = tuple(_resolve_int(s, env) for s in self.shape)
        return (np.zeros(shape), 0)

    def _dummy(self):
        shape = [1] + [int(s) if isinstance(s, (int, np.integer)) else 1 for s in self.shape[1:]]
        return (np.zeros(shape), 0)


class OffsetView(Node):
    """``v[start]``. Indexing a view again re-bases it (``v[a][b]`` is ``v[b]``): the
    symmetryPlane BC offsets an already offset normals view (BCs.py:38, 123), and only this
    reading keeps its normals on its own faces."""
    def __init__(self, base, start):
        super().__init__()
        self.base = base
        self.start = start

    def __getitem__(self, start):
        return OffsetView(self.base, start)

    @property
    def shape(self):
        return self.base.shape

    def _eval(self, env):
        arr, off = env.value(self.base)
        return (arr, off + _resolve_int(self.start, env))

    def _dummy(self):
        return self.base._dummy()


class KernelOutput(Node):
    def __init__(self, call, index, dummy, shape=None):
        super().__init__()
        self.call = call
        self.index = index
        self.dummy = dummy
        # an output written into a given array has that array's shape (a reduction into a
        # Zeros((1, 1)) is (1, 1)); otherwise one row per element of the range
        self.shape = tuple(shape) if shape is not None else (None,) + tuple(dummy[0].shape[1:])

    def _eval(self, env):
        return env.kernel(self.call)[self.index]

    def _dummy(self):
        return self.dummy


class _Env(object):
    def __init__(self, feed):
        self.feed = feed
        self.cache = {}
        self.kcache = {}

    def value(self, node):
        if node in self.cache:
            return self.cache[node]
        v = node._eval(self)
        self.cache[node] = v
        return v

    def kernel(self, call):
        if call.uid not in self.kcache:
            self.kcache[call.uid] = call.run(self)
        return self.kcache[call.uid]


# ---------------------------------------------------------------- element tensors

class Tensor(object):
    """Values of one kernel argument/expression over the element range: shape (n,)+eshape."""
    __array_ufunc__ = None
    __array_priority__ = 1000

    def __init__(self, value=None, full=None, off=0, n=None):
        if isinstance(value, tuple) and isinstance(full, list):
            # Tensor(shape, [elements]): an element tensor assembled from scalars per element
            # (postpro.py:564-612 builds 5x5 matrices so), constants broadcast to the rows
            shape, elems = value, full
            vals = [np.asarray(Tensor._v(e), np.float64) for e in elems]
            rows = max([v.shape[0] for v in vals if v.ndim >= 1] + [1])
            cols = [np.broadcast_to(v.reshape(-1, 1) if v.ndim else np.full((1, 1), float(v)), (rows, 1))
                    for v in vals]
            value = np.concatenate(cols, axis=1).reshape((rows,) + tuple(shape))
            full, off, n = None, 0, None
        self._value = value
        self.full = full
        self.off = off
        self.n = n

    @property
    def value(self):
        if self._value is None:
            self._value = self.full[self.off:self.off + self.n]
            if len(self._value) != self.n:
                raise IndexError('kernel range exceeds array rows')
        return self._value

    @property
    def shape(self):
        return tuple(self.value.shape[1:])

    # -- construction helpers
    @staticmethod
    def _v(x):
        return x.value if isinstance(x, Tensor) else x

    @staticmethod
    def _align(a, b):
        if isinstance(a, Tensor) and isinstance(b, Tensor):
            va, vb = a.value, b.value
            if va.ndim < vb.ndim and va.shape[1:] == (1,):
                va = va.reshape(va.shape[:1] + (1,) * (vb.ndim - 1))
            elif vb.ndim < va.ndim and vb.shape[1:] == (1,):
                vb = vb.reshape(vb.shape[:1] + (1,) * (va.ndim - 1))
            return va, vb
        return Tensor._v(a), Tensor._v(b)

    def _bin(self, other, op, reverse=False):
        a, b = (other, self) if reverse else (self, other)
        va, vb = Tensor._align(a, b)
        return Tensor(op(va, vb))

    def __add__(self, o): return self._bin(o, np.add)
    def __radd__(self, o): return self._bin(o, np.add, True)
    def __sub__(self, o): return self._bin(o, np.subtract)
    def __rsub__(self, o): return self._bin(o, np.subtract, True)
    def __mul__(self, o): return self._bin(o, np.multiply)
    def __rmul__(self, o): return self._bin(o, np.multiply, True)
    def __truediv__(self, o): return self._bin(o, np.true_divide)
    def __rtruediv__(self, o): return self._bin(o, np.true_divide, True)
    def __lt__(self, o): return self._bin(o, np.less)
    def __gt__(self, o): return self._bin(o, np.greater)
    def __neg__(self): return Tensor(-self.value)
    def __abs__(self): return Tensor(np.abs(self.value))
    def __pow__(self, p): return Tensor(np.power(self.value, p))

    def sqrt(self):
        return Tensor(np.sqrt(self.value))

    def __getitem__(self, i):
        v = self.value[(slice(None),) + i] if isinstance(i, tuple) else self.value[:, i]
        if v.ndim == 1:
            v = v.reshape(-1, 1)
        return Tensor(v)

    def __setitem__(self, i, t):
        v = np.array(self.value, copy=True)
        tv = Tensor._v(t)
        if v[:, i].ndim == 1:
            v[:, i] = np.asarray(tv).reshape(-1)
        else:
            v[:, i] = tv
        self._value = v

    # -- tensor algebra: products summed left to right
    def dot(self, o):
        a, b = self.value, Tensor._v(o)
        if a.ndim == 3:     # (n, m, 3) . (n, 3) -> (n, m)
            out = a[:, :, 0] * b[:, None, 0]
            for k in range(1, a.shape[2]):
                out = out + a[:, :, k] * b[:, None, k]
            return Tensor(out)
        out = a[:, 0] * b[:, 0]
        for k in range(1, a.shape[1]):
            out = out + a[:, k] * b[:, k]
        return Tensor(out.reshape(-1, 1))

    def magSqr(self):
        return self.dot(self)

    def tensordot(self, o):
        return self.dot(o)

    def outer(self, o):
        a, b = self.value, Tensor._v(o)
        return Tensor(a[:, :, None] * b[:, None, :])

    def transpose(self):
        return Tensor(np.ascontiguousarray(np.swapaxes(self.value, 1, 2)))

    def trace(self):
        v = self.value
        out = v[:, 0, 0]
        for k in range(1, v.shape[1]):
            out = out + v[:, k, k]
        return Tensor(out.reshape(-1, 1))

    def stabilise(self, s):
        v = self.value
        return Tensor(np.where(v < 0, v - s, v + s))

    # -- kernel-argument access
    def extract(self, idx):
        iv = Tensor._v(idx).reshape(-1).astype(np.int64)
        return Tensor(self.full[self.off + iv])

    def index(self):
        return Tensor(self.value)

    def scalar(self):
        row = self.full[self.off]
        return Tensor(np.broadcast_to(row, (self.n,) + row.shape).copy())

    # -- reductions over the element range
    def sum(self):
        v = self.value
        return _Reduce(np.cumsum(v, axis=0)[-1:])

    def reduce_max(self):
        return _Reduce(np.max(self.value, axis=0, keepdims=True))

    def reduce_sum(self):
        return self.sum()

    @staticmethod
    def collate(*args):
        return _Collate([(Tensor._v(args[k]), Tensor._v(args[k + 1])) for k in range(0, len(args), 2)])

    @staticmethod
    def switch(cond, a, b):
        c, va = Tensor._align(cond, a)
        c2, vb = Tensor._align(cond, b)
        return Tensor(np.where(c if np.ndim(c) >= np.ndim(c2) else c2, va, vb))

    @staticmethod
    def max(a, b):
        va, vb = Tensor._align(a, b)
        return Tensor(np.maximum(va, vb))


class _Reduce(Tensor):
    pass


class _Collate(object):
    def __init__(self, pairs):
        self.pairs = pairs


# ---------------------------------------------------------------- kernels and functions

class KernelCall(Node):
    def __init__(self, func, n, outputs, args, kwargs):
        super().__init__()
        self.func, self.n, self.outputs, self.args_, self.kwargs = func, n, outputs, args, kwargs

    def _tensors(self, env, n, dummy=False):
        ts = []
        for a in self.args_:
            if isinstance(a, Node):
                v = a._dummy() if dummy else env.value(a)
                if isinstance(v, tuple):
                    arr, off = v
                    ts.append(Tensor(full=arr, off=off, n=n))
                else:
                    ts.append(v)
            else:
                ts.append(a)
        return ts

    def _apply(self, results, outs, n):
        if not isinstance(results, (tuple, list)):
            results = (results,)
        produced = []
        for k, r in enumerate(results):
            if outs is not None:
                arr, off = outs[k]
                arr = np.array(arr, copy=True)
                if isinstance(r, _Collate) and len(r.pairs[0][0]) == 0:
                    pass
                elif isinstance(r, _Collate):
                    nrows = len(r.pairs[0][0])
                    m = len(r.pairs)
                    vals = np.stack([np.asarray(p[0]).reshape(nrows, -1) for p in r.pairs], axis=1)
                    idx = np.stack([np.asarray(p[1]).reshape(nrows) for p in r.pairs], axis=1)
                    flat = arr.reshape(arr.shape[0], -1)
                    np.add.at(flat, off + idx.reshape(-1).astype(np.int64), vals.reshape(nrows * m, -1))
                    arr = flat.reshape(arr.shape)
                elif isinstance(r, _Reduce):
                    arr[off] = np.asarray(r.value).reshape(arr[off].shape)
                else:
                    v = Tensor._v(r)
                    v = np.broadcast_to(v, (n,) + v.shape[1:]) if np.ndim(v) else np.full((n,), v)
                    arr[off:off + n] = v.reshape((n,) + arr.shape[1:])
                produced.append((arr, 0))
            else:
                v = np.asarray(Tensor._v(r))
                if not isinstance(r, _Reduce):
                    v = np.broadcast_to(v, (n,) + v.shape[1:]).copy() if v.ndim else np.full((n, 1), v)
                produced.append((v, 0))
        return produced

    def dry(self):
        ts = self._tensors(None, 1, dummy=True)
        with np.errstate(all='ignore'):
            res = self.func(*ts, **self.kwargs)
        outs = None if self.outputs is None else [o._dummy() for o in self.outputs]
        single = not isinstance(res, (tuple, list))
        return single, self._apply(res, outs, 1)

    def run(self, env):
        if self.n is None:
            # no range given: the rows of the first array argument
            arr, off = next(env.value(a) for a in self.args_ if isinstance(a, Node))
            n = arr.shape[0] - off
        else:
            n = _resolve_int(self.n, env)
        ts = self._tensors(env, n)
        res = self.func(*ts, **self.kwargs)
        outs = None if self.outputs is None else [env.value(o) for o in self.outputs]
        return self._apply(res, outs, n)


class Kernel(object):
    def __init__(self, func):
        self.func = func

    def __call__(self, n=None, outputs=None):
        def call(*args, **kwargs):
            kc = KernelCall(self.func, n, outputs, args, kwargs)
            single, dummies = kc.dry()
            shapes = [getattr(o, 'shape', None) for o in outputs] if outputs else [None] * len(dummies)
            outs = tuple(KernelOutput(kc, k, d, shapes[k] if k < len(shapes) else None)
                         for k, d in enumerate(dummies))
            # one result is returned bare (BCs.py:65-71, density.py:410 use it so)
            if len(outs) == 1:
                return outs[0]
            return outs
        return call


class ExternalNode(Node):
    """Output k of a compiled external operation, computed when the graph is evaluated."""
    def __init__(self, fn, inputs, k, shape):
        super().__init__()
        self.fn = fn
        self.inputs = inputs
        self.k = k
        self.shape = shape

    def _eval(self, env):
        key = ('ext', id(self.fn))
        if key not in env.cache:
            vals = []
            for x in self.inputs:
                arr, off = env.value(x)
                vals.append(np.asarray(arr)[off:])
            env.cache[key] = self.fn(*vals)
        return (env.cache[key][self.k], 0)

    def _dummy(self):
        return (np.zeros([1] + [int(s) if isinstance(s, (int, np.integer)) else 1 for s in self.shape[1:]]), 0)


# compiled external operations other than the one-rank MPI ones: name -> fn(*input arrays) ->
# output arrays; registered by the test infrastructure that restates them
EXTERNAL = {}


class ExternalFunctionOp(object):
    """MPI halo / allreduce ops on one rank: a halo op's outputs are the given output arrays
    unchanged (its call sites pass the field itself as its output); an allreduce over one rank
    is its inputs (objectives/vane.py:108-110 passes fresh zeros as the outputs). Other names
    are looked up in EXTERNAL."""
    def __init__(self, name, inputs, outputs, empty=False):
        self.name = name
        if name in EXTERNAL:
            fn = EXTERNAL[name]
            ins = tuple(inputs)

            def run(*vals):
                return fn(*vals)
            self.outputs = tuple(ExternalNode(run, ins, k, getattr(o, 'shape', None)) for k, o in enumerate(outputs))
        else:
            self.outputs = tuple(inputs) if name == 'mpi_allreduce' else tuple(outputs)


def ConstantOp(value=0.0):
    """A constant element (postpro.py:562)."""
    return float(value)


class Function(object):
    _functions = []

    def __init__(self, name, inputs, outputs, io_map=None, **kwargs):
        self.name = name
        self._inputs = list(inputs)
        self._outputs = list(outputs)
        Function._functions.append(self)

    def __call__(self, *values, **options):
        if len(values) != len(self._inputs):
            raise ValueError('%s: expected %d inputs, got %d' % (self.name, len(self._inputs), len(values)))
        env = _Env(dict(zip(self._inputs, values)))
        out = []
        for o in self._outputs:
            v = env.value(o)
            arr, off = v
            out.append(np.array(arr[off:], copy=True))
        return out

    def grad(self, *args, **kwargs):
        raise NotImplementedError('reverse mode is not part of the stand-in')

    @classmethod
    def createCodeDir(cls, *args, **kwargs):
        pass

    @classmethod
    def compile(cls, *args, **kwargs):
        pass

    @classmethod
    def initialize(cls, *args, **kwargs):
        pass
