"""ctypes binding of ``libafvm.so`` (declarations in include/afvm.h).

The library is the only compute path: importing this module raises if it has not been
built, and nothing falls back to a CPU implementation.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libafvm.so')

AFVM_OK, AFVM_ERR_BAD_ARG, AFVM_ERR_OOM, AFVM_ERR_NONFINITE, AFVM_ERR_TIMEOUT, \
    AFVM_ERR_CUDA, AFVM_ERR_UNSUPPORTED = range(7)
STATUS_NAMES = {0: 'OK', 1: 'BAD_ARG', 2: 'OOM', 3: 'NONFINITE', 4: 'TIMEOUT', 5: 'CUDA', 6: 'UNSUPPORTED'}

AFVM_FP64, AFVM_FP32, AFVM_FP32_STATE64 = 0, 1, 2
AFVM_PATCH_PLAIN, AFVM_PATCH_CYCLIC, AFVM_PATCH_PROCESSOR = 0, 1, 2
AFVM_BC_ZERO_GRADIENT, AFVM_BC_FIXED_VALUE, AFVM_BC_SYMMETRY_PLANE, AFVM_BC_CYCLIC, AFVM_BC_CBC_UPT, \
    AFVM_BC_CBC_TOTAL_PT = range(6)
AFVM_RIEMANN_ROE, AFVM_RIEMANN_LF = 0, 1
AFVM_MU_CONSTANT, AFVM_MU_SUTHERLAND = 0, 1
AFVM_OBJ_NONE, AFVM_OBJ_KINETIC_ENERGY, AFVM_OBJ_DRAG, AFVM_OBJ_SUM_T, AFVM_OBJ_VANE = range(5)
AFVM_VISC = {'uniform': 1, 'turkel': 2, 'abarbanel': 3}

_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int32)
_v = C.c_void_p


class Patch(C.Structure):
    _fields_ = [('startFace', C.c_int32), ('nFaces', C.c_int32), ('kind', C.c_int32),
                ('neighbourPatch', C.c_int32)]


class MeshIn(C.Structure):
    _fields_ = [('nPoints', C.c_int32), ('points', _d), ('nFaces', C.c_int32), ('faces', _i),
                ('nInternalFaces', C.c_int32), ('owner', _i), ('neighbour', _i),
                ('nInternalCells', C.c_int32), ('nPatches', C.c_int32), ('patches', C.POINTER(Patch))]


class MeshOut(C.Structure):
    _fields_ = [('normals', _d), ('faceCentres', _d), ('areas', _d), ('cellCentres', _d),
                ('volumes', _d), ('neighbour', _i), ('deltas', _d), ('deltasUnit', _d),
                ('weights', _d), ('linearWeights', _d), ('quadraticWeights', _d),
                ('cellFaces', _i), ('cellOwner', _i), ('cellNeighbours', _i),
                ('cellNeighboursMatOp', _i), ('nLocalCells', C.c_int32)]


class MeshTensors(C.Structure):
    _fields_ = [('areas', _d), ('volumesL', _d), ('volumesR', _d), ('weights', _d), ('deltas', _d),
                ('normals', _d), ('deltasUnit', _d), ('linearWeights', _d), ('quadraticWeights', _d),
                ('volumes', _d), ('owner', _i), ('neighbour', _i), ('cellFaces', _i),
                ('cellNeighbours', _i), ('cellOwner', _i),
                ('nCells', C.c_int32), ('nFaces', C.c_int32), ('nInternalCells', C.c_int32),
                ('nInternalFaces', C.c_int32), ('nLocalCells', C.c_int32), ('nRemoteCells', C.c_int32),
                ('nLocalFaces', C.c_int32), ('nGhostCells', C.c_int32),
                ('nPatches', C.c_int32), ('patches', C.POINTER(Patch))]


class PatchBC(C.Structure):
    _fields_ = [('U', C.c_int32), ('T', C.c_int32), ('p', C.c_int32),
                ('U_value', _d), ('T_value', _d), ('p_value', _d)]


class Physics(C.Structure):
    _fields_ = [('gamma', C.c_double), ('Cp', C.c_double), ('Pr', C.c_double),
                ('mu_model', C.c_int32), ('mu0', C.c_double), ('mu_As', C.c_double), ('mu_Ts', C.c_double),
                ('riemann', C.c_int32), ('boundary_riemann', C.c_int32),
                ('objective', C.c_int32), ('objective_patch', C.c_int32)]


class ObjectiveVane(C.Structure):
    _fields_ = [('nPlaneCells', C.c_int32), ('planeCells', C.POINTER(C.c_int32)), ('planeAreas', _d),
                ('normal', C.c_double * 3), ('ptin', C.c_double), ('nHeatPatches', C.c_int32),
                ('heatPatches', C.POINTER(C.c_int32)), ('heatWeights', C.POINTER(_d)), ('Tw', C.c_double),
                ('a', C.c_double), ('b', C.c_double)]


class ParamGrad(C.Structure):
    _fields_ = [('areas', _d), ('volumesL', _d), ('volumesR', _d), ('weights', _d), ('deltas', _d),
                ('normals', _d), ('deltasUnit', _d), ('linearWeights', _d), ('quadraticWeights', _d),
                ('volumes', _d), ('bcPatch', C.c_int32), ('bcField', C.c_int32), ('bc', _d)]


# name -> (restype, argtypes); every symbol declared in include/afvm.h
SIGNATURES = {
    'afvm_mesh_build': (C.c_int, [C.POINTER(MeshIn), C.POINTER(MeshOut)]),
    'afvm_mesh_build_device': (C.c_int, [C.POINTER(MeshIn), C.POINTER(MeshOut), _v]),
    'afvm_mesh_reorder_device': (C.c_int, [C.POINTER(MeshIn), _i, _i, _i, _i, _i, _i, _v]),
    'afvm_ctx_create': (C.c_int, [C.POINTER(MeshTensors), C.POINTER(PatchBC), C.POINTER(Physics),
                                  C.c_int32, C.c_int32, C.POINTER(_v)]),
    'afvm_ctx_destroy': (C.c_int, [_v]),
    'afvm_last_error': (C.c_char_p, [_v]),
    'afvm_ctx_precision': (C.c_int, [_v]),
    'afvm_ctx_device_bytes': (C.c_int64, [_v]),
    'afvm_set_bc_value': (C.c_int, [_v, C.c_int32, C.c_int32, _d]),
    'afvm_set_gauge': (C.c_int, [_v, C.c_double, C.c_double, C.c_double]),
    'afvm_get_gauge': (C.c_int, [_v, _d]),
    'afvm_set_objective_vane': (C.c_int, [_v, C.POINTER(ObjectiveVane)]),
    'afvm_set_objective_sink': (C.c_int, [_v, _v]),
    'afvm_set_objective_seed': (C.c_int, [_v, _v]),
    'afvm_primal_step': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v, _d, _d, _v]),
    'afvm_primal_step_stages': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v, _v, _d, _d, _v]),
    'afvm_primal_step_host': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v, _d, _d, _v]),
    'afvm_primal_run': (C.c_int, [_v, _v, _v, _v, C.c_int32, C.c_double, C.c_double, C.c_double,
                                  C.c_int32, _v, _v, _v, _d, _d, _d, _v]),
    'afvm_adjoint_step': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v,
                                    C.c_double, C.c_double, _v, _v, _v, _v, _v, _v, _v]),
    'afvm_adjoint_step_stages': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v, _v,
                                           C.c_double, C.c_double, _v, _v, _v, _v, _v, _v, _v]),
    'afvm_tape_elements': (C.c_int64, [_v]),
    'afvm_primal_step_tape': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v, _v, _v,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double), _v]),
    'afvm_adjoint_step_tape': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v, _v, _v,
                                         C.c_double, C.c_double, _v, _v, _v, _v, _v, _v, _v]),
    'afvm_adjoint_step_params': (C.c_int, [_v, _v, _v, _v, C.c_double, _v, _v, _v, _v, _v, _v, _v, _v,
                                           C.c_double, C.c_double, _v, _v, _v, _v, _v, _v,
                                           C.POINTER(ParamGrad), _v]),
    'afvm_sensitivity': (C.c_int, [_v, C.c_int32, C.POINTER(_d), C.POINTER(_d),
                                   C.POINTER(C.c_int64), _d, _v]),
    'afvm_adjoint_energy': (C.c_int, [_v, _v, _v, _v, _v, _v, _v, _d, _v]),
    'afvm_boundary_values': (C.c_int, [_v, _v, _v, _v, _v, _v]),
    'afvm_adjoint_viscosity': (C.c_int, [_v, _v, _v, _v, C.c_int32, C.c_double, C.c_double, _v, _v, _v, _d, _d,
                                         C.POINTER(C.c_int32), _v]),
    'afvm_profile': (C.c_int, [_v, C.c_int32]),
    'afvm_profile_read': (C.c_int, [_v, C.c_int32, _d, C.POINTER(C.c_int64)]),
    'afvm_profile_kernel_name': (C.c_char_p, [C.c_int32]),
    'afvm_fma_peak': (C.c_int, [C.c_int32, C.c_int32, _d]),
    'afvm_sensitivity_noalloc': (C.c_int, [C.c_int32, C.c_int32, C.POINTER(_d), C.POINTER(_d),
                                           C.POINTER(C.c_int64), _d, _v]),
    'afvm_copy_to_device': (C.c_int, [C.c_int32, _v, C.c_int32, _v, C.c_int32, C.c_int64, _v]),
    'afvm_copy_to_host': (C.c_int, [C.c_int32, _v, C.c_int32, _v, C.c_int32, C.c_int64, _v]),
}


def fma_peak(device=0, fp64=True):
    v = C.c_double()
    check(lib().afvm_fma_peak(device, 1 if fp64 else 0, C.byref(v)), None, 'afvm_fma_peak')
    return v.value


def kernel_names():
    out = []
    k = 0
    while True:
        n = lib().afvm_profile_kernel_name(k)
        if not n:
            return out
        out.append(n.decode())
        k += 1

_lib = None


class AfvmError(RuntimeError):
    def __init__(self, status, message):
        super().__init__('afvm status %s: %s' % (STATUS_NAMES.get(status, status), message))
        self.status = status


def lib():
    """The loaded native library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError('libafvm.so not built (%s); run adfvm_gb300.build.build()' % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, ctx=None, what=''):
    if status != AFVM_OK:
        msg = what
        if ctx is not None:
            m = lib().afvm_last_error(ctx)
            if m:
                msg = (what + ': ' if what else '') + m.decode()
        raise AfvmError(status, msg)


def to_device(a, t):
    """Host array `a` (numpy, float64 or float32, any host memory) into the CUDA tensor `t`
    (same number of values, float64 or float32), converted when the types differ; ordered on
    t's device's current stream (afvm_copy_to_device)."""
    import numpy as np
    import torch
    a = np.ascontiguousarray(a)
    if (a.dtype not in (np.float64, np.float32) or t.dtype not in (torch.float64, torch.float32)
            or a.size != t.numel() or not t.is_contiguous() or t.device.type != 'cuda'):
        raise ValueError('to_device: %s array of %d values into a %s tensor of %d' % (a.dtype, a.size, t.dtype, t.numel()))
    stream = torch.cuda.current_stream(t.device).cuda_stream
    check(lib().afvm_copy_to_device(t.device.index, C.c_void_p(t.data_ptr()), t.element_size(),
                                    C.c_void_p(a.ctypes.data), a.itemsize, a.size, C.c_void_p(stream)),
          None, 'afvm_copy_to_device')
    return t


def to_host(t, out):
    """The CUDA tensor `t` (float64 or float32) into the numpy array `out` (float64 or float32,
    C-contiguous, same number of values), converted when the types differ; returns once `out`
    holds the values (afvm_copy_to_host)."""
    import numpy as np
    import torch
    t = t.contiguous()
    if (out.dtype not in (np.float64, np.float32) or t.dtype not in (torch.float64, torch.float32)
            or out.size != t.numel() or not out.flags['C_CONTIGUOUS'] or t.device.type != 'cuda'):
        raise ValueError('to_host: %s tensor of %d values into a %s array of %d' % (t.dtype, t.numel(), out.dtype, out.size))
    stream = torch.cuda.current_stream(t.device).cuda_stream
    check(lib().afvm_copy_to_host(t.device.index, C.c_void_p(out.ctypes.data), out.itemsize,
                                  C.c_void_p(t.data_ptr()), t.element_size(), out.size, C.c_void_p(stream)),
          None, 'afvm_copy_to_host')
    return out


def dptr(a):
    """double* of a C-contiguous float64 numpy array."""
    assert a.dtype.name == 'float64' and a.flags['C_CONTIGUOUS']
    return a.ctypes.data_as(_d)


def iptr(a):
    assert a.dtype.name == 'int32' and a.flags['C_CONTIGUOUS']
    return a.ctypes.data_as(_i)
