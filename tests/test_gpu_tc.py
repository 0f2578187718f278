"""tcgen05 tensor-core path (16-bit B): parity with the oracle.

Bit tiles are expanded to exact 0/1 BF16/FP16 operands and products by 1 are
exact, so integer-valued B must give identical results; for N(0,1) B the
FP32 accumulation order differs from the oracle's, and every element is
checked against FP64 relative to its summation scale (≤ 1e-4), well inside
the 1e-2 bound of the precision form."""
import os

import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import bf16_dev, words_dev

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture
def force_tc():
    old = os.environ.get("BSP_TC")
    os.environ["BSP_TC"] = "1"
    yield
    if old is None:
        del os.environ["BSP_TC"]
    else:
        os.environ["BSP_TC"] = old


def _b16(Bf, kind):
    if kind == "bf16":
        b = W.f32_to_bf16_bits(Bf)
        return bf16_dev(b), W.bf16_bits_to_f32(b)
    t = torch.from_numpy(Bf).half().cuda()
    return t, t.float().cpu().numpy()


@pytest.mark.parametrize("kind", ["bf16", "f16"])
@pytest.mark.parametrize("M,K,N,p", [(128, 32, 256, 0.3), (300, 200, 264, 0.2), (1000, 1000, 512, 0.05),
                                     (77, 64, 8, 0.5), (512, 2048, 1024, 0.01)])
def test_tc_random(force_tc, kind, M, K, N, p):
    rng = np.random.default_rng(M + K + N)
    bits = rng.random((M, K)) < p
    if K >= 128:
        bits[: min(M, 130), 64:128] = False  # K tiles 2-3 empty for the first row block
    words = W.pack_bits(bits)
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    Bf = rng.standard_normal((K, N)).astype(np.float32)
    B, Bexact = _b16(Bf, kind)
    C = ops.spmm(wd, K, B, plan=plan).cpu().numpy()
    assert capi.device_status() == 0
    mx, mean, _ = O.rel_errors(C, O.spmm_f64(words, K, Bexact), O.spmm_abs_f64(words, K, Bexact))
    assert mx <= TOL, (mx, mean)
    # integer-valued B: exact
    Bi = rng.integers(-8, 9, (K, N)).astype(np.float32)
    Bt, Bie = _b16(Bi, kind)
    Ci = ops.spmm(wd, K, Bt, plan=plan).cpu().numpy()
    assert np.array_equal(Ci.astype(np.float64), O.spmm_f64(words, K, Bie))


def test_tc_block_structured_sample():
    """Block-structured A (32x32 tiles present w.p. 0.3, bits 0.8), the
    tensor-core workload at a reduced size, through the default dispatch."""
    A, present = W.block_bits(2048, 4096, p_tile=0.3, p_bit=0.8, seed=5)
    words = W.pack_bits(A)
    wd = words_dev(words)
    plan = ops.Plan(wd, 4096)
    rng = np.random.default_rng(6)
    Bf = rng.standard_normal((4096, 768)).astype(np.float32)
    B, Bexact = _b16(Bf, "bf16")
    C = ops.spmm(wd, 4096, B, plan=plan).cpu().numpy()
    assert capi.device_status() == 0
    mx, _, _ = O.rel_errors(C, O.spmm_f64(words, 4096, Bexact), O.spmm_abs_f64(words, 4096, Bexact))
    assert mx <= TOL
    # the CUDA-core walk agrees
    os.environ["BSP_TC"] = "0"
    try:
        C2 = ops.spmm(wd, 4096, B, plan=plan).cpu().numpy()
    finally:
        del os.environ["BSP_TC"]
    assert np.abs(C - C2).max() <= 1e-4 * max(1.0, np.abs(C2).max())


@pytest.mark.slow
def test_config3_full_size_row_sample():
    cfg = W.config3()
    words, K, N = cfg["words"], cfg["K"], cfg["N"]
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    B = bf16_dev(cfg["B"])
    C = ops.spmm(wd, K, B, plan=plan)
    assert capi.device_status() == 0
    Bexact = W.bf16_bits_to_f32(cfg["B"])
    rows = np.r_[0:128, 8192:8256, 16320:16384]
    Cs = C[torch.from_numpy(rows).cuda()].cpu().numpy()
    C64 = O.spmm_f64(words[rows], K, Bexact)
    mx, _, mxn = O.rel_errors(Cs, C64, O.spmm_abs_f64(words[rows], K, Bexact))
    assert mx <= TOL and mxn <= 1e-2


@pytest.mark.parametrize("M,K,N,p", [(512, 8192, 256, 0.3), (300, 4096, 40, 0.1), (256, 16384, 512, 0.02)])
def test_tc_split_k(force_tc, M, K, N, p):
    # few output tiles and a long reduction: with the preferred workspace the
    # occupied K tiles are split over several CTAs and the partials added in
    # a fixed order; the minimum workspace keeps one CTA per output tile
    rng = np.random.default_rng(M + K)
    words = W.pack_bits(rng.random((M, K)) < p)
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    assert plan.workspace_bytes(N) > plan.workspace_bytes(N, preferred=False)
    Bi = rng.integers(-8, 9, (K, N)).astype(np.float32)
    Bt, Bie = _b16(Bi, "bf16")
    ref = O.spmm_f64(words, K, Bie)
    C1 = ops.spmm(wd, K, Bt, plan=plan).cpu().numpy()  # split
    ws0 = torch.empty(max(plan.workspace_bytes(N, preferred=False), 1), dtype=torch.uint8, device="cuda")
    C0 = ops.spmm(wd, K, Bt, plan=plan, workspace=ws0).cpu().numpy()  # no split
    assert capi.device_status() == 0
    assert np.array_equal(C1.astype(np.float64), ref) and np.array_equal(C0.astype(np.float64), ref)
    # N(0,1) B: both orders within the precision-form tolerance, split run to run identical
    Bf = rng.standard_normal((K, N)).astype(np.float32)
    B, Bexact = _b16(Bf, "bf16")
    Ca = ops.spmm(wd, K, B, plan=plan).cpu().numpy()
    Cb = ops.spmm(wd, K, B, plan=plan).cpu().numpy()
    assert np.array_equal(Ca, Cb)
    mx, _, _ = O.rel_errors(Ca, O.spmm_f64(words, K, Bexact), O.spmm_abs_f64(words, K, Bexact))
    assert mx <= TOL, mx


@pytest.mark.parametrize("M,K,N", [(300, 200, 264), (1000, 1000, 512), (513, 4096, 776), (64, 40, 8),
                                   (8200, 300, 72), (600, 8300, 40)])
def test_tiled_b_matches_tensor_boxes(force_tc, M, K, N):
    # the preferred workspace copies B (and G) into tile order, one bulk copy
    # per tile, where the output has many row blocks; the minimum keeps TMA
    # tensor boxes.  The shared-memory bytes are the same, so integer-valued
    # operands (exact in any order) give identical results, including ragged
    # edges (K and M tails, a last column block of 8 or 8 < n < 64 columns);
    # N(0,1) operands stay within the precision-form tolerance either way.
    rng = np.random.default_rng(M + 3 * K + N)
    bits = rng.random((M, K)) < 0.2
    words = W.pack_bits(bits)
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    ws_pref = torch.empty(plan.workspace_bytes(N), dtype=torch.uint8, device="cuda")
    ws_min = torch.empty(max(plan.workspace_bytes(N, preferred=False), 1), dtype=torch.uint8, device="cuda")
    Bi, Bie = _b16(rng.integers(-8, 9, (K, N)).astype(np.float32), "bf16")
    ref = O.spmm_f64(words, K, Bie)
    for ws in (ws_pref, ws_min):
        assert np.array_equal(ops.spmm(wd, K, Bi, plan=plan, workspace=ws).cpu().numpy().astype(np.float64), ref)
    B, Bexact = _b16(rng.standard_normal((K, N)).astype(np.float32), "bf16")
    for ws in (ws_pref, ws_min):
        C = ops.spmm(wd, K, B, plan=plan, workspace=ws).cpu().numpy()
        mx, _, _ = O.rel_errors(C, O.spmm_f64(words, K, Bexact), O.spmm_abs_f64(words, K, Bexact))
        assert mx <= TOL
    assert capi.device_status() == 0
    # transposed product: G [M][N] tiled over M
    n_min, n_pref = _t_workspaces(M, K, N)
    Gi, Gie = _b16(rng.integers(-8, 9, (M, N)).astype(np.float32), "bf16")
    ref_t = O.spmm_t_f64(words, M, K, Gie)
    for nb in (n_pref, n_min):
        ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
        dX = ops.spmm_t(wd, M, K, Gi, plan=plan, workspace=ws).cpu().numpy()
        assert np.array_equal(dX.astype(np.float64), ref_t)
    assert capi.device_status() == 0


def _t_workspaces(M, K, N):
    import ctypes
    a, b = ctypes.c_size_t(), ctypes.c_size_t()
    capi.call("bsp_spmm_t_workspace", M, K, ctypes.byref(a))
    capi.call("bsp_spmm_t_workspace_preferred", M, K, N, ctypes.byref(b))
    assert b.value >= a.value
    return a.value, b.value


@pytest.mark.parametrize("kind", ["bf16", "f16"])
@pytest.mark.parametrize("M,K,N,p", [(8200, 1000, 264, 0.05), (8448, 3000, 64, 0.01)])
def test_three_tile_stages(force_tc, kind, M, K, N, p):
    # 32+ row blocks: stages of three K tiles (two stages in flight); list
    # lengths that are not multiples of three leave a short last stage
    rng = np.random.default_rng(M + K)
    bits = rng.random((M, K)) < p
    bits[:300, 96:320] = False  # a run of empty K tiles for the first row blocks
    words = W.pack_bits(bits)
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    Bi, Bie = _b16(rng.integers(-8, 9, (K, N)).astype(np.float32), kind)
    C = ops.spmm(wd, K, Bi, plan=plan).cpu().numpy()
    assert capi.device_status() == 0
    assert np.array_equal(C.astype(np.float64), O.spmm_f64(words, K, Bie))
    B, Bexact = _b16(rng.standard_normal((K, N)).astype(np.float32), kind)
    C = ops.spmm(wd, K, B, plan=plan).cpu().numpy()
    mx, _, _ = O.rel_errors(C, O.spmm_f64(words, K, Bexact), O.spmm_abs_f64(words, K, Bexact))
    assert mx <= TOL
