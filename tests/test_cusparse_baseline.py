"""cuSPARSE's CSR SpMM, the reference's library baseline
(source/src/main.cu:1061-1131): its library loads and validates arguments
without a GPU, the CSR built from packed words matches the host conversion,
and on the GPU it computes the same C as the bitmap SpMM (bit-exact for
integer-valued FP32 B: every partial sum is an exact small integer)."""
import ctypes as C

import numpy as np
import pytest
import torch

from bitwise_spgemm_gb300 import cusparse_baseline as CS
from bitwise_spgemm_gb300 import workloads as W


def _need_lib():
    ok, why = CS.available()
    if not ok:
        pytest.skip(why)
    return CS._load()


def test_library_loads_and_rejects_bad_arguments():
    L = _need_lib()
    ms, first = C.c_float(), C.c_float()
    # M = 0, null pointers, bad dtype: refused before any CUDA call
    assert L.bsp_cusparse_spmm_csr(0, 4, 4, 0, None, None, None, None, 0, 4, None, 4, 0, 0, 1, None,
                                   C.byref(ms), C.byref(first)) == -1
    assert L.bsp_cusparse_spmm_csr(4, 4, 4, 1, None, None, None, None, 0, 4, None, 4, 0, 0, 1, None,
                                   C.byref(ms), C.byref(first)) == -1
    assert L.bsp_cusparse_spmm_csr(4, 4, 4, 0, 8, None, None, 8, 0, 2, 8, 4, 0, 0, 1, None,
                                   C.byref(ms), C.byref(first)) == -1  # ldb < N
    assert L.bsp_cusparse_spmm_csr(4, 4, 4, 0, 8, None, None, 8, 1, 4, 8, 4, 0, 0, 1, None,
                                   C.byref(ms), C.byref(first)) == -4  # FP16 not offered


@pytest.mark.parametrize("M,K", [(1, 1), (37, 70), (256, 1000)])
def test_csr_from_words_matches_host_conversion(M, K):
    rng = np.random.default_rng(M + K)
    bits = rng.random((M, K)) < 0.2
    words = W.pack_bits(bits)
    off, cols = CS.csr_from_words(torch.from_numpy(words.view(np.int32)), K)
    ro, co = W.bits_to_csr(words, M, K)
    assert np.array_equal(off.numpy(), ro) and np.array_equal(cols.numpy(), co)


@pytest.mark.gpu
def test_cusparse_matches_bitmap_spmm_integer_b():
    _need_lib()
    from bitwise_spgemm_gb300 import ops
    cfg = W.config1()
    M, K, N = cfg["M"], cfg["K"], cfg["N"]
    words = torch.from_numpy(np.ascontiguousarray(cfg["words"]).view(np.int32)).cuda()
    B = torch.from_numpy(cfg["B"]).cuda()
    ours = ops.spmm(words, K, B)
    off, cols = CS.csr_from_words(words, K)
    assert int(off[-1]) == int(np.unpackbits(cfg["words"].view(np.uint8)).sum())
    Cc, ms, first = CS.spmm_csr(off, cols, B, M, warmup=1, iters=2)
    assert ms > 0 and first > 0
    assert torch.equal(Cc, ours)


@pytest.mark.gpu
def test_cusparse_bf16_within_tolerance_or_refused():
    _need_lib()
    from bitwise_spgemm_gb300 import ops
    rng = np.random.default_rng(3)
    M, K, N = 300, 512, 128
    bits = rng.random((M, K)) < 0.1
    words = torch.from_numpy(W.pack_bits(bits).view(np.int32)).cuda()
    B = torch.from_numpy(rng.standard_normal((K, N), dtype=np.float32)).cuda().to(torch.bfloat16)
    ours = ops.spmm(words, K, B)
    off, cols = CS.csr_from_words(words, K)
    try:
        Cc, _, _ = CS.spmm_csr(off, cols, B, M, warmup=0, iters=1)
    except RuntimeError as exc:  # cuSPARSE does not offer BF16 in, FP32 out
        assert "status -4" in str(exc)
        return
    ref = bits.astype(np.float64) @ B.float().cpu().numpy().astype(np.float64)
    err = np.abs(Cc.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 1e-2
    assert (Cc - ours).abs().max().item() / ours.abs().max().item() < 1e-2
