"""ctypes wrapper around the C oracle — test infrastructure only.

Each function takes and returns numpy arrays and calls the restatement in
``bsp_oracle.c`` (which cites the reference file:line it follows).
"""
import ctypes as C

import numpy as np

from . import build as _build

_lib = None

DTYPE_CODES = {np.dtype(np.float32): 0, np.dtype(np.float16): 1,
               np.dtype(np.int8): 3, np.dtype(np.uint8): 4}
BF16_CODE = 2

_P = C.c_void_p
_I64 = C.c_int64
_I = C.c_int


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        sigs = {
            "orc_pack_rows": (_I, [_P, _I, _I64, _I64, _I64, _P, _I]),
            "orc_pack_cols": (_I, [_P, _I, _I64, _I64, _I64, _P, _I]),
            "orc_transpose_bits": (None, [_P, _I64, _I64, _P]),
            "orc_unpack_rows_f32": (None, [_P, _I64, _I64, _P, _I64, _I]),
            "orc_bitplanes": (_I, [_P, _I64, _I64, _I64, _I, _P, _I]),
            "orc_group_rows": (_I, [_P, _I64, _I64, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "orc_group_to_dense": (None, [_P, _P, _P, _I64, _I64, _I, _I, _P, _I64]),
            "orc_spmm_f64": (None, [_P, _I64, _I64, _P, _I64, _I64, _P, _I64]),
            "orc_spmm_abs_f64": (None, [_P, _I64, _I64, _P, _I64, _I64, _P, _I64]),
            "orc_spmm_f32": (None, [_P, _I64, _I64, _P, _I64, _I64, _P, _I64]),
            "orc_spmm_f32_mt": (None, [_P, _I64, _I64, _P, _I64, _I64, _P, _I64, _I]),
            "orc_spmm_t_f64": (None, [_P, _I64, _I64, _P, _I64, _I64, _P, _I64]),
            "orc_sddmm_f64": (None, [_P, _I64, _I64, _P, _I64, _P, _I64, _I64, _P]),
            "orc_dense_check_sum": (None, [_P, _P, _P, _I, _I, _I]),
            "orc_check": (_I64, [_P, _P, _P, _I, _I, _I]),
            "orc_dense_check_sum_mt": (None, [_P, _P, _P, _I, _I, _I, _I, _I, _I]),
            "orc_symbolic_rows": (None, [_P, _I64, _I64, _P, _I64, _P]),
            "orc_bitplane_spmm_f64": (None, [_P, _I64, _I64, _I64, _P, _I64, _I64, _P, _I64]),
            "orc_rows_to_tiles8": (_I64, [_P, _I64, _I64, _P, _P, _P, _P]),
            "orc_tiles8_to_rows": (None, [_P, _P, _P, _I64, _I64, _I64, _P]),
            "orc_csr_to_tiled": (None, [_P, _P, _P, _I64, _I64, _I, _I, _P, _P, _P, _P]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dtype=None):
    a = np.asarray(a) if dtype is None else np.asarray(a, dtype=dtype)
    return np.ascontiguousarray(a)


def kw(k):
    return (k + 31) // 32


def pack_rows(dense, msb_first=False, bf16=False):
    """Restates dense2bitmask (source/src/main.cu:591-628). ``dense`` is a 2-D
    numpy array; ``bf16=True`` means a uint16 array holding bfloat16 bits."""
    dense = _c(dense)
    M, K = dense.shape
    code = BF16_CODE if bf16 else DTYPE_CODES[dense.dtype]
    out = np.zeros((M, kw(K)), np.uint32)
    rc = lib().orc_pack_rows(_ptr(dense), code, M, K, K, _ptr(out), int(msb_first))
    assert rc == 0
    return out


def pack_cols(dense, msb_first=False, bf16=False):
    dense = _c(dense)
    M, K = dense.shape
    code = BF16_CODE if bf16 else DTYPE_CODES[dense.dtype]
    out = np.zeros((K, kw(M)), np.uint32)
    rc = lib().orc_pack_cols(_ptr(dense), code, M, K, K, _ptr(out), int(msb_first))
    assert rc == 0
    return out


def transpose_bits(words, M, K):
    words = _c(words, np.uint32)
    out = np.zeros((K, kw(M)), np.uint32)
    lib().orc_transpose_bits(_ptr(words), M, K, _ptr(out))
    return out


def unpack_rows(words, M, K, msb_first=False):
    words = _c(words, np.uint32)
    out = np.zeros((M, K), np.float32)
    lib().orc_unpack_rows_f32(_ptr(words), M, K, _ptr(out), K, int(msb_first))
    return out


def bitplanes(values, planes=8, msb_first=False):
    """Restates uint8_layout_trans (backup/layout_trans.cu:87-97), packed."""
    v = _c(values).view(np.uint8)
    M, K = v.shape
    out = np.zeros((planes, M, kw(K)), np.uint32)
    rc = lib().orc_bitplanes(_ptr(v), M, K, K, planes, _ptr(out), int(msb_first))
    assert rc == 0
    return out


def group_rows(words, tile_rows, max_groups):
    """Restates generate_groups_large (source/src/main.cu:50-247) serialised in
    ascending row order.  Returns a dict of numpy arrays."""
    words = _c(words, np.uint32)
    M, Kw = words.shape
    T = ((M + tile_rows - 1) // tile_rows) * Kw
    out = dict(
        group_id=np.zeros((M, Kw), np.int32),
        group_mask=np.zeros((T, max_groups), np.uint32),
        group_row=np.zeros((T, max_groups, 32), np.int32),
        spill_cnt=np.zeros(T, np.int32),
        spill_nnz=np.zeros(T, np.int32),
        spill_rows=np.zeros((T, tile_rows), np.int32),
        grouped_nnz=np.zeros(1, np.int64),
    )
    rc = lib().orc_group_rows(_ptr(words), M, Kw, tile_rows, max_groups,
                              _ptr(out["group_id"]), _ptr(out["group_mask"]),
                              _ptr(out["group_row"]), _ptr(out["spill_cnt"]),
                              _ptr(out["spill_nnz"]), _ptr(out["spill_rows"]),
                              _ptr(out["grouped_nnz"]))
    assert rc == 0
    return out


def group_to_dense(group_values, group_id, words, M, K, tile_rows, max_groups, dense=None):
    gv = _c(group_values, np.float32)
    gid = _c(group_id, np.int32)
    words = _c(words, np.uint32)
    out = np.zeros((M, K), np.float32) if dense is None else _c(dense, np.float32).copy()
    lib().orc_group_to_dense(_ptr(gv), _ptr(gid), _ptr(words), M, K, tile_rows,
                             max_groups, _ptr(out), K)
    return out


def spmm_f64(words, K, B):
    words = _c(words, np.uint32)
    B = _c(B, np.float32)
    M = words.shape[0]
    N = B.shape[1]
    out = np.zeros((M, N), np.float64)
    lib().orc_spmm_f64(_ptr(words), M, K, _ptr(B), N, N, _ptr(out), N)
    return out


def spmm_abs_f64(words, K, B):
    words = _c(words, np.uint32)
    B = _c(B, np.float32)
    M = words.shape[0]
    N = B.shape[1]
    out = np.zeros((M, N), np.float64)
    lib().orc_spmm_abs_f64(_ptr(words), M, K, _ptr(B), N, N, _ptr(out), N)
    return out


def spmm_f32(words, K, B, threads=1):
    words = _c(words, np.uint32)
    B = _c(B, np.float32)
    M = words.shape[0]
    N = B.shape[1]
    out = np.zeros((M, N), np.float32)
    if threads > 1:
        lib().orc_spmm_f32_mt(_ptr(words), M, K, _ptr(B), N, N, _ptr(out), N, threads)
    else:
        lib().orc_spmm_f32(_ptr(words), M, K, _ptr(B), N, N, _ptr(out), N)
    return out


def spmm_t_f64(words, M, K, G):
    words = _c(words, np.uint32)
    G = _c(G, np.float32)
    N = G.shape[1]
    out = np.zeros((K, N), np.float64)
    lib().orc_spmm_t_f64(_ptr(words), M, K, _ptr(G), N, N, _ptr(out), N)
    return out


def sddmm_f64(words, M, K, G, X):
    words = _c(words, np.uint32)
    G = _c(G, np.float32)
    X = _c(X, np.float32)
    N = G.shape[1]
    nnz = int(np.unpackbits(words.view(np.uint8)).sum())
    out = np.zeros(nnz, np.float64)
    lib().orc_sddmm_f64(_ptr(words), M, K, _ptr(G), N, _ptr(X), N, N, _ptr(out))
    return out


def dense_check_sum(A, B, threads=1, rows=None):
    """The reference CPU path, check()'s triple loop
    (backup/bit_wise_gemm.cu:13-32), on dense float A and B."""
    A = _c(A, np.float32)
    B = _c(B, np.float32)
    m, k = A.shape
    n = B.shape[1]
    out = np.zeros((m, n), np.float32)
    if threads > 1 or rows is not None:
        r0, r1 = (0, m) if rows is None else rows
        lib().orc_dense_check_sum_mt(_ptr(A), _ptr(B), _ptr(out), m, n, k, r0, r1, threads)
    else:
        lib().orc_dense_check_sum(_ptr(A), _ptr(B), _ptr(out), m, n, k)
    return out


def check(A, B, Cm):
    """check() of backup/bit_wise_gemm.cu:13-32: -1 when every element is within
    relative 1e-5, else the flat index of the first failing element."""
    A = _c(A, np.float32)
    B = _c(B, np.float32)
    Cm = _c(Cm, np.float32)
    m, k = A.shape
    n = B.shape[1]
    return int(lib().orc_check(_ptr(A), _ptr(B), _ptr(Cm), m, n, k))


def symbolic_rows(a_words, K, b_words, N):
    a_words = _c(a_words, np.uint32)
    b_words = _c(b_words, np.uint32)
    M = a_words.shape[0]
    out = np.zeros((M, kw(N)), np.uint32)
    lib().orc_symbolic_rows(_ptr(a_words), M, K, _ptr(b_words), N, _ptr(out))
    return out


def bitplane_spmm_f64(A_i8, B):
    A = _c(A_i8, np.int8)
    B = _c(B, np.float32)
    M, K = A.shape
    N = B.shape[1]
    out = np.zeros((M, N), np.float64)
    lib().orc_bitplane_spmm_f64(_ptr(A), M, K, K, _ptr(B), N, N, _ptr(out), N)
    return out


def rows_to_tiles8(words, M, K):
    """-> (bmp uint64[n], tile_row int32[n], tile_col int32[n], offset int32[n+1])."""
    words = _c(words, np.uint32)
    T = ((M + 7) // 8) * ((K + 7) // 8)
    bmp = np.zeros(T, np.uint64)
    tr = np.zeros(T, np.int32)
    tc = np.zeros(T, np.int32)
    off = np.zeros(T + 1, np.int32)
    n = int(lib().orc_rows_to_tiles8(_ptr(words), M, K, _ptr(bmp), _ptr(tr), _ptr(tc), _ptr(off)))
    return bmp[:n], tr[:n], tc[:n], off[: n + 1]


def tiles8_to_rows(bmp, tile_row, tile_col, M, K):
    bmp = _c(bmp, np.uint64)
    tr = _c(tile_row, np.int32)
    tc = _c(tile_col, np.int32)
    out = np.zeros((M, kw(K)), np.uint32)
    lib().orc_tiles8_to_rows(_ptr(bmp), _ptr(tr), _ptr(tc), len(bmp), M, K, _ptr(out))
    return out


def csr_to_tiled(row_ptr, col, val, M, K, tile_rows, tile_cols):
    """-> (tile_nnz_acc [T+1], tiled_offset [T, tile_rows+1], tiled_col [nnz], tiled_val [nnz])."""
    rp = _c(row_ptr, np.int32)
    cl = _c(col, np.int32)
    vl = _c(val, np.float32)
    T = ((M + tile_rows - 1) // tile_rows) * ((K + tile_cols - 1) // tile_cols)
    nnz = len(cl)
    acc = np.zeros(T + 1, np.int32)
    toff = np.zeros((T, tile_rows + 1), np.int32)
    tcol = np.zeros(max(nnz, 1), np.int32)
    tval = np.zeros(max(nnz, 1), np.float32)
    lib().orc_csr_to_tiled(_ptr(rp), _ptr(cl), _ptr(vl), M, K, tile_rows, tile_cols, _ptr(acc), _ptr(toff),
                           _ptr(tcol), _ptr(tval))
    return acc, toff, tcol[:nnz], tval[:nnz]


def rel_errors(C, C64, Cabs=None):
    """Error of C against the FP64 oracle.  Returns
    (max_scaled, mean_scaled, max_norm) where scaled = |C-C64| / (|A||B|)_ij
    (the FP32 summation bound's scale; entries with zero scale must be exact)
    and max_norm = max|C-C64| / max|C64|."""
    C = np.asarray(C, np.float64)
    err = np.abs(C - C64)
    max_norm = float(err.max() / max(np.abs(C64).max(), 1e-300)) if err.size else 0.0
    if Cabs is None:
        return None, None, max_norm
    scale = np.where(Cabs > 0, Cabs, 1.0)
    scaled = np.where(Cabs > 0, err / scale, err)
    return float(scaled.max()) if scaled.size else 0.0, float(scaled.mean()) if scaled.size else 0.0, max_norm
