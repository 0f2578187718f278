"""Autotuner on the GPU: bsp_tune times the schedules, leaves C correct and
caches the fastest for the shape bucket; bsp_spmm then runs the cached
schedule (seen through its results: each engine is deterministic and the
tensor cores round FP32 sums differently from the CUDA cores)."""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import bf16_dev, words_dev

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(autouse=True)
def clean_cache():
    capi.lib().bsp_tune_cache_clear()
    yield
    capi.lib().bsp_tune_cache_clear()


def test_tune_prototype_plan_fp32():
    A, _, _ = W.clustered_bits(2048, 2048, n_proto=16)
    words = W.pack_bits(A)
    wd = words_dev(words)
    plan = ops.Plan(wd, 2048, mode=capi.PLAN_PROTO)
    assert plan.info()["mode"] == capi.PLAN_PROTO
    B = np.random.default_rng(4).standard_normal((2048, 256), dtype=np.float32)
    Bt = torch.from_numpy(B).cuda()
    C = torch.empty(2048, 256, device="cuda")
    best = ops.tune(wd, 2048, Bt, plan, out=C)
    assert best["engine"] == 2 and best["ms"] > 0 and 0 <= best["proto_variant"] <= 8
    mx, _, _ = O.rel_errors(C.cpu().numpy(), O.spmm_f64(words, 2048, B), O.spmm_abs_f64(words, 2048, B))
    assert mx <= 1e-5
    n = __import__("ctypes").c_int(0)
    capi.lib().bsp_tune_cache_size(__import__("ctypes").byref(n))
    assert n.value == 1
    C2 = ops.spmm(wd, 2048, Bt, plan=plan).cpu().numpy()  # the cached schedule
    assert np.array_equal(C2, C.cpu().numpy())


def test_dispatch_follows_the_cache(tmp_path, monkeypatch):
    rng = np.random.default_rng(11)
    bits, _ = W.block_bits(1024, 2048, p_tile=0.3)
    words = W.pack_bits(bits)
    wd = words_dev(words)
    plan = ops.Plan(wd, 2048)
    Bb = W.f32_to_bf16_bits(rng.standard_normal((2048, 512), dtype=np.float32))
    B = bf16_dev(Bb)
    ops.tune(wd, 2048, B, plan)
    path = tmp_path / "cache.json"
    assert capi.lib().bsp_tune_cache_save(str(path).encode()) == 0
    text = path.read_text()
    ref = {}
    for tc in ("0", "1"):
        monkeypatch.setenv("BSP_TC", tc)
        ref[tc] = ops.spmm(wd, 2048, B, plan=plan).cpu().numpy()
    monkeypatch.delenv("BSP_TC")
    assert not np.array_equal(ref["0"], ref["1"])  # the two engines round differently
    import re
    n = __import__("ctypes").c_int(0)
    for engine, want in ((2, "0"), (1, "1")):
        path.write_text(re.sub(r'"engine": \d', '"engine": %d' % engine, text))
        assert capi.lib().bsp_tune_cache_load(str(path).encode(), __import__("ctypes").byref(n)) == 0
        got = ops.spmm(wd, 2048, B, plan=plan).cpu().numpy()
        assert np.array_equal(got, ref[want]), engine


def test_cache_file_written_through_env(tmp_path):
    # a fresh process with BSP_TUNE_CACHE: tuning writes the file, a second
    # process reads it back at first use
    path = tmp_path / "tune.json"
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import numpy as np, torch, ctypes as C\n"
        "from bitwise_spgemm_gb300 import ops, capi, workloads as W\n"
        "A = np.random.default_rng(1).random((512, 1024)) < 0.05\n"
        "wd = torch.from_numpy(W.pack_bits(A).view(np.int32)).cuda()\n"
        "plan = ops.Plan(wd, 1024)\n"
        "B = torch.randn(1024, 128, device='cuda')\n"
        "if sys.argv[1] == 'tune': ops.tune(wd, 1024, B, plan)\n"
        "n = C.c_int(0); capi.lib().bsp_tune_cache_size(C.byref(n)); print('entries', n.value)\n" % ROOT)
    env = dict(os.environ, BSP_TUNE_CACHE=str(path))
    r = subprocess.run([sys.executable, "-c", code, "tune"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert path.exists() and '"bsp_tune_cache": 2' in path.read_text()
    r2 = subprocess.run([sys.executable, "-c", code, "read"], env=env, capture_output=True, text=True, timeout=300)
    assert r2.returncode == 0 and "entries 1" in r2.stdout, r2.stdout + r2.stderr


@pytest.mark.parametrize("M", [512, 8192])
def test_tensor_core_tile_forms_from_the_cache(M, tmp_path):
    """Each tensor-core tile form a cache entry can name (2 or 3 K tiles per
    stage, B by boxes or pre-tiled, split-K by the rule or never) gives the
    product within the tensor-core tolerance of FP64; tuning picks one of
    them and records it.  512 rows: the split-K rule applies; 8192 rows:
    B is pre-tiled by the rule."""
    import ctypes
    import re
    rng = np.random.default_rng(M)
    K, N = 2048, 256
    bits, _ = W.block_bits(M, K, p_tile=0.3)
    words = W.pack_bits(bits)
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    Bf = rng.standard_normal((K, N), dtype=np.float32)
    Bb = W.f32_to_bf16_bits(Bf)
    B, Bx = bf16_dev(Bb), W.bf16_bits_to_f32(Bb)
    C64, Cabs = O.spmm_f64(words, K, Bx), O.spmm_abs_f64(words, K, Bx)
    best = ops.tune(wd, K, B, plan)
    if best["engine"] == 1:
        assert best["tc_stage_tiles"] in (2, 3) and best["tc_tiled_b"] in (0, 1) and best["tc_split"] in (-1, 0)
    path = tmp_path / "cache.json"
    assert capi.lib().bsp_tune_cache_save(str(path).encode()) == 0
    text = path.read_text()
    n = ctypes.c_int(0)
    for tps in (2, 3):
        for tiled in (0, 1):
            for split in (-1, 0):
                t = re.sub(r'"engine": \d', '"engine": 1', text)
                t = re.sub(r'"tc_tps": -?\d', '"tc_tps": %d' % tps, t)
                t = re.sub(r'"tc_tiled": -?\d', '"tc_tiled": %d' % tiled, t)
                t = re.sub(r'"tc_split": -?\d', '"tc_split": %d' % split, t)
                path.write_text(t)
                assert capi.lib().bsp_tune_cache_load(str(path).encode(), ctypes.byref(n)) == 0
                C = ops.spmm(wd, K, B, plan=plan).cpu().numpy()
                mx, _, _ = O.rel_errors(C, C64, Cabs)
                assert mx <= 1e-4, (tps, tiled, split, mx)
    assert capi.device_status() == 0
