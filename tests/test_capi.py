"""CPU-only checks of the C ABI library: it loads, exports every entry point
declared in include/bsp.h, and rejects bad arguments before touching a GPU."""
import ctypes as C
import os
import re

from bitwise_spgemm_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(bsp_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    names = declared_symbols()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(L, n), n
    assert set(capi.SIGNATURES) >= names


def test_status_strings_and_version():
    L = capi.lib()
    assert L.bsp_version() >= 100
    for st, name in capi.STATUS.items():
        assert L.bsp_status_string(st).decode().startswith(name)


def test_argument_validation_without_gpu():
    L = capi.lib()
    P = C.c_void_p
    fake = P(0x10000)
    # bad dtype / bit order / negative sizes / ld < K
    assert L.bsp_pack_rows(fake, 9, 4, 4, 4, fake, 0, None) == -1
    assert L.bsp_pack_rows(fake, 0, 4, 4, 4, fake, 2, None) == -1
    assert L.bsp_pack_rows(fake, 0, -1, 4, 4, fake, 0, None) == -1
    assert L.bsp_pack_rows(fake, 0, 4, 8, 4, fake, 0, None) == -1
    assert L.bsp_pack_rows(None, 0, 4, 8, 8, fake, 0, None) == -1
    # empty problems are no-ops
    assert L.bsp_pack_rows(None, 0, 0, 8, 8, None, 0, None) == 0
    # misaligned pointers
    assert L.bsp_pack_rows(P(0x10001), 0, 4, 8, 8, fake, 0, None) == -2
    # grouping limits
    assert L.bsp_group_rows(fake, 4, 1, 0, 2, fake, fake, None, None, None, None, None, None) == -1
    assert L.bsp_group_rows(fake, 4, 1, 8, 33, fake, fake, None, None, None, None, None, None) == -1
    # spmm: unsupported B dtype, ld < N, capacity
    assert L.bsp_spmm(fake, 4, 32, fake, 3, 8, 8, fake, 8, None, None, 0, None) == -4
    assert L.bsp_spmm(fake, 4, 32, fake, 0, 4, 8, fake, 8, None, None, 0, None) == -1
    assert L.bsp_spmm(fake, 4, 1 << 40, fake, 0, 8, 8, fake, 8, None, None, 0, None) == -8
    # output side and multi-bit operands
    assert L.bsp_symbolic_rows(fake, 4, 32, fake, -1, fake, None) == -1
    assert L.bsp_symbolic_rows(fake, 4, 32, fake, 64, None, None) == -1
    assert L.bsp_symbolic_rows(P(0x10002), 4, 32, fake, 64, fake, None) == -2
    assert L.bsp_bitplane_spmm(fake, 0, 1, 4, 32, fake, 0, 8, 8, fake, 8, None) == -1
    assert L.bsp_bitplane_spmm(fake, 9, 1, 4, 32, fake, 0, 8, 8, fake, 8, None) == -1
    assert L.bsp_bitplane_spmm(fake, 8, 1, 4, 32, fake, 3, 8, 8, fake, 8, None) == -4
    assert L.bsp_bitplane_spmm(fake, 8, 1, 4, 32, fake, 0, 4, 8, fake, 8, None) == -1
    ws = C.c_size_t(0)
    assert L.bsp_spmm_i8_workspace(3, 33, C.byref(ws)) == 0 and ws.value == 4 * 8 * 3 * 2 + 256
    assert L.bsp_spmm_i8(fake, 3, 33, 40, fake, 0, 8, 8, fake, 8, None, 0, None) == -3
    assert L.bsp_spmm_i8(fake, 3, 33, 32, fake, 0, 8, 8, fake, 8, fake, 1 << 20, None) == -1
    # gradient batch: null out-pointer, unsupported dtype, N not a multiple of 8
    assert L.bsp_batch_grad_create(None, 0, 8, 2, None, None) == -1
    h = C.c_void_p()
    assert L.bsp_batch_grad_create(None, 0, 8, 0, C.byref(h), None) == -4
    assert L.bsp_batch_grad_create(None, 0, 12, 2, C.byref(h), None) == -2
    assert L.bsp_batched_spmm_grad(None, None) == -1
    # batch tuner: null batch or out-pointers
    shape, ms = C.c_int(), C.c_float()
    assert L.bsp_batch_tune(None, None, C.byref(shape), C.byref(ms)) == -1
    # L2 gather probe: slice size, alignment, warp count
    assert L.bsp_probe_gather(fake, 8, 2048, fake, 8, 4, 384, fake, None) == -1
    assert L.bsp_probe_gather(P(0x10004), 8, 2048, fake, 8, 4, 512, fake, None) == -2
    assert L.bsp_probe_gather(fake, 8, 2048, fake, 12, 4, 512, fake, None) == -1
    # plan handles
    assert L.bsp_plan_destroy(None) == 0
    assert L.bsp_plan_destroy_async(None, None) == 0
    assert L.bsp_plan_get_info(None, None) == -1
    n = C.c_size_t(7)
    assert L.bsp_spmm_workspace(None, 16, C.byref(n)) == 0 and n.value == 0
