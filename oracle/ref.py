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
        }.items():
            getattr(L, n).argtypes = a
            getattr(L, n).restype = C.c_int
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
