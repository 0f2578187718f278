"""ctypes binding of the C ABI in include/bsp.h (libbsp.so).

There is no fallback: if ``libbsp.so`` is missing the first call raises.
Functions here take raw integers (device pointers, sizes, stream handles)
exactly as the C ABI does; ``ops.py`` adds torch-tensor conveniences.
"""
import ctypes as C
import os

from . import build as _build

BSP_OK = 0
STATUS = {
    0: "BSP_OK", -1: "BSP_ERR_INVALID_ARG", -2: "BSP_ERR_ALIGNMENT", -3: "BSP_ERR_WORKSPACE",
    -4: "BSP_ERR_UNSUPPORTED", -5: "BSP_ERR_CUDA", -6: "BSP_ERR_DEVICE_TIMEOUT",
    -7: "BSP_ERR_ALLOC", -8: "BSP_ERR_CAPACITY", -9: "BSP_ERR_QUEUE", -10: "BSP_ERR_INTERNAL",
}
F32, F16, BF16, I8, U8 = 0, 1, 2, 3, 4
LSB_FIRST, MSB_FIRST = 0, 1
PLAN_AUTO, PLAN_DIRECT, PLAN_PROTO = 0, 1, 2


class BspError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = "%s failed: %s" % (where, STATUS.get(status, status))
        if status == -5 and _lib is not None:
            msg += " (cudaError %d)" % _lib.bsp_last_cuda_error()
        super().__init__(msg)


class PlanParams(C.Structure):
    _fields_ = [("mode", C.c_int), ("signature_hashes", C.c_int),
                ("min_cluster_rows", C.c_int), ("seed", C.c_uint32)]


class PlanInfo(C.Structure):
    _fields_ = [("M", C.c_int64), ("K", C.c_int64), ("nnz", C.c_int64), ("mode", C.c_int),
                ("n_proto", C.c_int64), ("proto_nnz", C.c_int64), ("delta_nnz", C.c_int64),
                ("direct_rows", C.c_int64), ("direct_nnz", C.c_int64), ("occ_tiles", C.c_int64)]


class Schedule(C.Structure):
    _fields_ = [("engine", C.c_int), ("proto_path", C.c_int), ("proto_variant", C.c_int), ("ms", C.c_float),
                ("tc_stage_tiles", C.c_int), ("tc_tiled_b", C.c_int), ("tc_split", C.c_int)]


class Problem(C.Structure):
    _fields_ = [("A_words", C.c_void_p), ("M", C.c_int64), ("K", C.c_int64), ("B", C.c_void_p),
                ("ldb", C.c_int64), ("C", C.c_void_p), ("ldc", C.c_int64)]


class ProblemGrad(C.Structure):
    _fields_ = [("A_words", C.c_void_p), ("M", C.c_int64), ("K", C.c_int64), ("X", C.c_void_p),
                ("ldx", C.c_int64), ("G", C.c_void_p), ("ldg", C.c_int64), ("dX", C.c_void_p),
                ("lddx", C.c_int64), ("dA", C.c_void_p), ("ldda", C.c_int64)]


_P = C.c_void_p
_I64 = C.c_int64
_I = C.c_int
_SZ = C.c_size_t

# name -> argument types (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "bsp_status_string": [_I],
    "bsp_version": [],
    "bsp_last_cuda_error": [],
    "bsp_pack_rows": [_P, _I, _I64, _I64, _I64, _P, _I, _P],
    "bsp_pack_cols": [_P, _I, _I64, _I64, _I64, _P, _I, _P],
    "bsp_transpose_bits": [_P, _I64, _I64, _P, _P],
    "bsp_unpack_rows": [_P, _I64, _I64, _P, _I, _I64, _I, _P],
    "bsp_bitplanes": [_P, _I64, _I64, _I64, _I, _P, _I, _P],
    "bsp_group_rows": [_P, _I64, _I64, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P],
    "bsp_group_to_dense": [_P, _P, _P, _I64, _I64, _I, _I, _P, _I64, _P],
    "bsp_plan_create": [_P, _I64, _I64, C.POINTER(PlanParams), C.POINTER(_P), _P],
    "bsp_plan_destroy": [_P],
    "bsp_plan_destroy_async": [_P, _P],
    "bsp_plan_get_info": [_P, C.POINTER(PlanInfo)],
    "bsp_spmm_workspace": [_P, _I64, C.POINTER(_SZ)],
    "bsp_spmm": [_P, _I64, _I64, _P, _I, _I64, _I64, _P, _I64, _P, _P, _SZ, _P],
    "bsp_device_status": [C.POINTER(_I), _I],
    "bsp_spmm_t_workspace": [_I64, _I64, C.POINTER(_SZ)],
    "bsp_batch_create": [C.POINTER(Problem), _I, _I64, _I, C.POINTER(_P), _P],
    "bsp_batch_destroy": [_P],
    "bsp_batched_spmm": [_P, _P],
    "bsp_batch_tune": [_P, _P, C.POINTER(_I), C.POINTER(C.c_float)],
    "bsp_batch_grad_create": [C.POINTER(ProblemGrad), _I, _I64, _I, C.POINTER(_P), _P],
    "bsp_batched_spmm_grad": [_P, _P],
    "bsp_probe_gather": [_P, _I64, _I64, _P, _I64, _I64, _I, _P, _P],
    "bsp_spmm_t": [_P, _I64, _I64, _P, _I, _I64, _I64, _P, _I64, _P, _P, _SZ, _P],
    "bsp_sddmm": [_P, _I64, _I64, _P, _I64, _P, _I64, _I, _I64, _P, _I64, _P, _P],
    "bsp_symbolic_rows": [_P, _I64, _I64, _P, _I64, _P, _P],
    "bsp_symbolic_workspace": [_P, _I64, _P],
    "bsp_symbolic_rows_planned": [_P, _I64, _I64, _P, _I64, _P, _P, _P, _SZ, _P],
    "bsp_bitplane_spmm": [_P, _I, _I, _I64, _I64, _P, _I, _I64, _I64, _P, _I64, _P],
    "bsp_spmm_i8_workspace": [_I64, _I64, C.POINTER(_SZ)],
    "bsp_spmm_workspace_preferred": [_P, _I64, C.POINTER(_SZ)],
    "bsp_spmm_t_workspace_preferred": [_I64, _I64, _I64, C.POINTER(_SZ)],
    "bsp_tune": [_P, _I64, _I64, _P, _I, _I64, _I64, _P, _I64, _P, _P, _SZ, _P, C.POINTER(Schedule)],
    "bsp_tune_cache_load": [C.c_char_p, C.POINTER(_I)],
    "bsp_tune_cache_save": [C.c_char_p],
    "bsp_tune_cache_clear": [],
    "bsp_tune_cache_size": [C.POINTER(_I)],
    "bsp_bitplanes_rows": [_P, _I64, _I64, _I64, _I, _P, _P],
    "bsp_stack_planes_b": [_P, _I, _I64, _I64, _I64, _I, _I, _P, _I64, _P],
    "bsp_spmm_i8": [_P, _I64, _I64, _I64, _P, _I, _I64, _I64, _P, _I64, _P, _SZ, _P],
    "bsp_tiles8_workspace": [_I64, _I64, C.POINTER(_SZ)],
    "bsp_rows_to_tiles8": [_P, _I64, _I64, _P, _P, _P, _P, _P, _P, _SZ, _P],
    "bsp_tiles8_to_rows": [_P, _P, _P, _I64, _I64, _I64, _P, _P],
    "bsp_csr_to_tiled_workspace": [_I64, _I64, _I64, _I, _I, C.POINTER(_SZ)],
    "bsp_csr_to_tiled": [_P, _P, _P, _I, _I64, _I64, _I64, _I, _I, _P, _P, _P, _P, _P, _SZ, _P],
    "bsp_spmm_noalloc": [_P, _I64, _I64, _P, _I, _I64, _I64, _P, _I64, _P, _P],
}
_RESTYPES = {"bsp_status_string": C.c_char_p}

_lib = None


def lib_path():
    return _build.LIB


def lib():
    """Load libbsp.so (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            try:
                _build.build()
            except Exception as exc:  # no toolkit: fail loudly, no fallback
                raise RuntimeError("libbsp.so is missing and could not be built: %s" % exc)
        L = C.CDLL(path)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, C.c_int)
        _lib = L
    return _lib


def call(name, *args):
    st = getattr(lib(), name)(*args)
    if st != BSP_OK:
        raise BspError(st, name)
    return st


def device_status(clear=True):
    """Device error word of the asynchronous kernels (0 = none)."""
    v = C.c_int(0)
    call("bsp_device_status", C.byref(v), int(clear))
    return v.value
