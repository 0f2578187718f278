"""The autotuner's cache file, on CPU: entries load, a malformed file is
ignored as a whole (the cache keeps its contents), saving writes a complete
file through a temporary one and rename."""
import ctypes as C
import os

from bitwise_spgemm_gb300 import capi

GOOD = """{"bsp_tune_cache": 2, "entries": [
 {"key": "M13K13N9d9t0p2", "engine": 2, "proto_path": 0, "proto_variant": 4, "tc_tps": 0, "tc_tiled": -1, "tc_split": -1, "ms": 0.032800},
 {"key": "M14K14N11d4t2p1", "engine": 1, "proto_path": 0, "proto_variant": 0, "tc_tps": 3, "tc_tiled": 1, "tc_split": 0, "ms": 0.595000}
]}
"""
# a file in the first format (no tile form) is refused as a whole
OLD = """{"bsp_tune_cache": 1, "entries": [
 {"key": "M13K13N9d9t0p2", "engine": 2, "proto_path": 0, "proto_variant": 4, "ms": 0.032800}
]}
"""


def _size(L):
    n = C.c_int(-1)
    assert L.bsp_tune_cache_size(C.byref(n)) == 0
    return n.value


def test_cache_load_save_and_corrupt_files(tmp_path):
    L = capi.lib()
    good = tmp_path / "good.json"
    good.write_text(GOOD)
    n = C.c_int(0)
    assert L.bsp_tune_cache_load(str(good).encode(), C.byref(n)) == 0 and n.value == 2
    assert _size(L) == 2
    # malformed files: truncated, a bad engine, junk between entries
    for bad in (GOOD[: len(GOOD) // 2],
                GOOD.replace('"engine": 1', '"engine": 7'),
                GOOD.replace('"tc_tps": 3', '"tc_tps": 5'),
                GOOD.replace("]}", "garbage\n]}"),
                OLD):
        p = tmp_path / "bad.json"
        p.write_text(bad)
        assert L.bsp_tune_cache_load(str(p).encode(), C.byref(n)) == -1
        assert _size(L) == 2  # unchanged
    assert L.bsp_tune_cache_load(str(tmp_path / "missing.json").encode(), C.byref(n)) == -1
    out = tmp_path / "saved.json"
    assert L.bsp_tune_cache_save(str(out).encode()) == 0
    assert not [f for f in os.listdir(tmp_path) if ".tmp" in f]
    assert L.bsp_tune_cache_clear() == 0 and _size(L) == 0
    assert L.bsp_tune_cache_load(str(out).encode(), C.byref(n)) == 0 and n.value == 2
    assert out.read_text() == GOOD
    assert L.bsp_tune_cache_clear() == 0
