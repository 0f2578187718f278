"""ctypes access to the reference's own code built into oracle/_ref/ by
build_ref.py — used only to pin the oracle in tests (this container only;
the reference checkout is not available elsewhere)."""
import ctypes as C
import os

import numpy as np

from . import build_ref

_emu = None
_chk = None
_P = C.c_void_p


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def available():
    return (os.path.exists(os.path.join(build_ref.OUT, "libref_emu.so"))
            or build_ref.available())


def emu():
    global _emu
    if _emu is None:
        build_ref.build()
        L = C.CDLL(os.path.join(build_ref.OUT, "libref_emu.so"))
        for n, a in {
            "ref_dense2bitmask": [_P, C.c_int, C.c_int, C.c_int, _P],
            "ref_generate_groups_large": [_P, _P, C.c_int, C.c_int, C.c_int] + [_P] * 8,
            "ref_group2dense": [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int],
            "ref_uint8_layout_trans": [_P, C.c_int, C.c_int, _P],
            "ref_layout_trans": [_P, C.c_int, C.c_int, C.c_int, _P],
            "ref_uint8_spmm": [_P, _P, _P, C.c_int, C.c_int, C.c_int],
            "ref_csr2tiledcsr": [_P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int] + [_P] * 6,
            "ref_pre_spgemm": [_P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int] + [_P] * 6,
        }.items():
            getattr(L, n).argtypes = a
            getattr(L, n).restype = C.c_int
        L.ref_coo2bmp.argtypes = [_P, _P, _P, C.c_int64, C.c_int, C.c_int, C.c_int64] + [_P] * 5
        L.ref_coo2bmp.restype = C.c_int64
        _emu = L
    return _emu


def check_lib():
    global _chk
    if _chk is None:
        build_ref.build()
        path = os.path.join(build_ref.OUT, "libref_check.so")
        if not os.path.exists(path):
            return None
        L = C.CDLL(path)
        f = getattr(L, "_Z5checkPKfS0_S0_iii")
        f.argtypes = [_P, _P, _P, C.c_int, C.c_int, C.c_int]
        f.restype = C.c_bool
        _chk = f
    return _chk


def dense2bitmask(dense, tile_rows):
    d = np.ascontiguousarray(dense, np.float32)
    M, K = d.shape
    out = np.zeros((M, K // 32), np.int32)
    assert emu().ref_dense2bitmask(_ptr(d), M, K, tile_rows, _ptr(out)) == 0
    return out.view(np.uint32)


def generate_groups_large(words_msb, dense, tile_rows):
    w = np.ascontiguousarray(words_msb).view(np.int32)
    d = np.ascontiguousarray(dense, np.float32)
    M, K = d.shape
    T = (M // tile_rows) * (K // 32)
    o = dict(group_id=np.zeros((M, K // 32), np.int32), group_mask=np.zeros((T, 2), np.int32),
             group_val=np.zeros((T, 2, 32), np.int8), spill_cnt=np.zeros(T, np.int32),
             spill_nnz=np.zeros(T, np.int32), hash_table=np.zeros((T, 2048), np.int32),
             hash_table_rev=np.zeros((T, 2048), np.int32), nnz=np.zeros(1, np.int32))
    rc = emu().ref_generate_groups_large(_ptr(w), _ptr(d), M, K, tile_rows, _ptr(o["group_id"]),
                                         _ptr(o["group_mask"]), _ptr(o["group_val"]),
                                         _ptr(o["spill_cnt"]), _ptr(o["spill_nnz"]),
                                         _ptr(o["hash_table"]), _ptr(o["hash_table_rev"]),
                                         _ptr(o["nnz"]))
    assert rc == 0
    o["group_mask"] = o["group_mask"].view(np.uint32)
    return o


def group2dense(group_values, group_idx_tm, bitmask_tm, M, N, tile_rows, dense=None):
    gv = np.ascontiguousarray(group_values, np.float32)
    gi = np.ascontiguousarray(group_idx_tm, np.int32)
    bm = np.ascontiguousarray(bitmask_tm).view(np.int32)
    out = np.zeros((M, N), np.float32) if dense is None else np.array(dense, np.float32)
    assert emu().ref_group2dense(_ptr(gv), _ptr(out), _ptr(gi), _ptr(bm), M, N, tile_rows) == 0
    return out


def uint8_layout_trans(src):
    s = np.ascontiguousarray(src, np.uint8)
    m, k = s.shape
    out = np.zeros((8, m, k), np.int32)
    assert emu().ref_uint8_layout_trans(_ptr(s), m, k, _ptr(out)) == 0
    return out


def layout_trans(src_f32, bit_width=32):
    s = np.ascontiguousarray(src_f32, np.float32)
    m, k = s.shape
    out = np.zeros((bit_width, m, k), np.int32)
    assert emu().ref_layout_trans(_ptr(s), m, k, bit_width, _ptr(out)) == 0
    return out


def uint8_spmm(mask_planes, B):
    mk = np.ascontiguousarray(mask_planes, np.int32)
    Bf = np.ascontiguousarray(B, np.float32)
    _, m, k = mk.shape
    n = Bf.shape[1]
    out = np.zeros((m, n), np.float32)
    assert emu().ref_uint8_spmm(_ptr(mk), _ptr(Bf), _ptr(out), m, k, n) == 0
    return out


def check(A, B, Cm):
    f = check_lib()
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    Cm = np.ascontiguousarray(Cm, np.float32)
    m, k = A.shape
    n = B.shape[1]
    return bool(f(_ptr(A), _ptr(B), _ptr(Cm), m, n, k))


def csr2tiledcsr(row_ptr, col, val, M, K, tile_h, tile_w):
    """csr2tiledcsr (source/src/main.cu:499-588) with tiles tile_h x tile_w
    (64x64, 256x256 or 32x128).  -> dict of tile_nnz_acc [T+1], tile_nnz [T],
    tile_row_nnz [M, K/tile_w], tiled_offset [T, tile_h+1], tiled_col [nnz],
    tiled_val [nnz]."""
    rp = np.ascontiguousarray(row_ptr, np.int32)
    cl = np.ascontiguousarray(col, np.int32)
    vl = np.ascontiguousarray(val, np.float32)
    T = (M // tile_h) * (K // tile_w)
    nnz = len(cl)
    o = dict(tile_nnz_acc=np.zeros(T + 1, np.int32), tile_nnz=np.zeros(T, np.int32),
             tile_row_nnz=np.zeros((M, K // tile_w), np.int32),
             tiled_offset=np.zeros((T, tile_h + 1), np.int32),
             tiled_col=np.zeros(max(nnz, 1), np.int32), tiled_val=np.zeros(max(nnz, 1), np.float32))
    rc = emu().ref_csr2tiledcsr(_ptr(rp), _ptr(cl), _ptr(vl), M, K, tile_h, tile_w,
                                _ptr(o["tile_nnz_acc"]), _ptr(o["tile_nnz"]), _ptr(o["tile_row_nnz"]),
                                _ptr(o["tiled_offset"]), _ptr(o["tiled_col"]), _ptr(o["tiled_val"]))
    assert rc == 0
    o["tiled_col"] = o["tiled_col"][:nnz]
    o["tiled_val"] = o["tiled_val"][:nnz]
    return o


def pre_spgemm(b_words, tiled, M, K, N, tile):
    """pre_spgemm (source/src/transform.cuh:984-1157) with TILE_HEIGHT =
    SPLIT_K = tile = K.  b_words: B's row masks [K, N/32]; tiled: the dict of
    csr2tiledcsr for A with the same tile.  -> dict with c_bits and
    group_idx [M, N/32] (brought from the kernel's tile-major order to row
    order), group_mask [T, 2], spill_cnt/spill_nnz [T], nnz [1]."""
    bw = np.ascontiguousarray(b_words).view(np.int32)
    Nw = N // 32
    T = (M // tile) * Nw
    cb = np.zeros(M * Nw, np.int32)
    gi = np.zeros(M * Nw, np.int32)
    o = dict(group_mask=np.zeros((T, 2), np.int32), spill_cnt=np.zeros(T, np.int32),
             spill_nnz=np.zeros(T, np.int32), nnz=np.zeros(1, np.int32))
    toff = np.ascontiguousarray(tiled["tiled_offset"], np.int32)
    tcol = np.ascontiguousarray(tiled["tiled_col"], np.int32)
    acc = np.ascontiguousarray(tiled["tile_nnz_acc"], np.int32)
    rc = emu().ref_pre_spgemm(_ptr(bw), _ptr(toff), _ptr(tcol), _ptr(acc), M, K, N, tile,
                              _ptr(cb), _ptr(gi), _ptr(o["group_mask"]), _ptr(o["spill_cnt"]),
                              _ptr(o["spill_nnz"]), _ptr(o["nnz"]))
    assert rc == 0

    def rows(tm):  # (rb, w, r) tile-major -> [M, Nw]
        return tm.reshape(M // tile, Nw, tile).transpose(0, 2, 1).reshape(M, Nw)
    o["c_bits"] = rows(cb).view(np.uint32)
    o["group_idx"] = rows(gi)
    o["group_mask"] = o["group_mask"].view(np.uint32)
    return o


def coo2bmp(row, col, val, M, K):
    """coo2bmp_noTuple_d (source/src/main.cu:692-779) on Thrust's sequential
    back end.  -> (bmp uint64[n], tile_row int32[n], tile_col int32[n],
    idx uint32[n] (exclusive popcount scan), elems float32[nnz])."""
    r = np.ascontiguousarray(row, np.int32)
    c = np.ascontiguousarray(col, np.int32)
    v = np.ascontiguousarray(val, np.float32)
    nnz = len(r)
    cap = max(nnz, 1)
    bmp = np.zeros(cap, np.uint64)
    tr = np.zeros(cap, np.int32)
    tc = np.zeros(cap, np.int32)
    ix = np.zeros(cap, np.uint32)
    el = np.zeros(cap, np.float32)
    n = int(emu().ref_coo2bmp(_ptr(r), _ptr(c), _ptr(v), nnz, M, K, cap, _ptr(bmp), _ptr(tr),
                              _ptr(tc), _ptr(ix), _ptr(el)))
    assert n >= 0
    return bmp[:n], tr[:n], tc[:n], ix[:n], el[:nnz]
