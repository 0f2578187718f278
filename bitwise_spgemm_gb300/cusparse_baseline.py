"""cuSPARSE's CSR SpMM, the reference's library baseline (reference
source/src/main.cu:1061-1131, ``timing_cusparse_spmm_csr``), for timing
beside the bitmap SpMM and for cross-checking its results.  It lives in its
own ``libbsp_cusparse.so``; nothing in the bitmap library calls it.

``csr_from_words`` builds the CSR form of a packed bit matrix on the GPU
with torch (setup, not timed); ``spmm_csr`` runs and times cuSPARSE.
"""
import ctypes as C
import os

import torch

from . import build as _build

BSP_F32, BSP_BF16 = 0, 2
ALG_DEFAULT = 0  # CUSPARSE_SPMM_ALG_DEFAULT, as the reference

_lib = None
_why = None


def _load():
    global _lib, _why
    if _lib is None and _why is None:
        path = _build.CUSPARSE_LIB
        if not os.path.exists(path) and _build.build_cusparse_baseline() is None:
            _why = "libbsp_cusparse.so could not be built (no cuSPARSE in the toolkit)"
            return None
        try:
            L = C.CDLL(path)
        except OSError as exc:
            _why = "libbsp_cusparse.so does not load: %s" % exc
            return None
        fn = L.bsp_cusparse_spmm_csr
        fn.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                       C.c_void_p, C.c_int, C.c_int64, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int,
                       C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        fn.restype = C.c_int
        _lib = L
    return _lib


def available():
    """(True, "") when the baseline library loads, else (False, reason)."""
    return (_load() is not None, _why or "")


def csr_from_words(words, K):
    """Packed rows [M, ceil(K/32)] (int32 on the GPU, LSB = lowest column) ->
    (row offsets int32 [M+1], column indices int32 [nnz]) on the GPU."""
    M, Kw = words.shape
    shifts = torch.arange(32, device=words.device, dtype=torch.int32)
    bits = ((words.unsqueeze(-1) >> shifts) & 1).view(M, Kw * 32)[:, :K].bool()
    offsets = torch.zeros(M + 1, dtype=torch.int32, device=words.device)
    offsets[1:] = bits.sum(1).cumsum(0).to(torch.int32)
    cols = bits.nonzero()[:, 1].to(torch.int32).contiguous()
    return offsets, cols


def spmm_csr(offsets, cols, B, M, out=None, alg=ALG_DEFAULT, warmup=2, iters=5):
    """C = A·B by cuSPARSE for the 0/1 matrix A in CSR (values 1 in B's dtype,
    FP32 or BF16), FP32 C.  Returns (C, warm ms per call, the reference-style
    cold call's ms).  Raises RuntimeError when cuSPARSE refuses the
    combination or the library is missing."""
    L = _load()
    if L is None:
        raise RuntimeError(_why)
    if B.dtype not in (torch.float32, torch.bfloat16) or B.stride(1) != 1:
        raise ValueError("B must be row-major FP32 or BF16")
    K, N = B.shape
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device=B.device)
    vals = torch.ones(cols.numel(), dtype=B.dtype, device=B.device)
    ms, first = C.c_float(), C.c_float()
    st = L.bsp_cusparse_spmm_csr(M, K, N, cols.numel(), offsets.data_ptr(), cols.data_ptr(), vals.data_ptr(),
                                 B.data_ptr(), BSP_F32 if B.dtype == torch.float32 else BSP_BF16, B.stride(0),
                                 out.data_ptr(), out.stride(0), alg, warmup, iters,
                                 torch.cuda.current_stream().cuda_stream, C.byref(ms), C.byref(first))
    if st != 0:
        raise RuntimeError("cuSPARSE SpMM failed: status %d" % st)
    return out, ms.value, first.value
