"""bsp_spmm_noalloc — the SpMM entry point that allocates nothing.

Callers that may not allocate device memory when they run the SpMM (plugin
callbacks handed only pointers, hot loops that must not call the allocator,
processes whose device memory belongs to another allocator) call this entry
point; its scratch is a fixed 8 MiB device array inside the library.  This
test calls it through the C ABI twice in a row and compares each result with
the ordinary workspace entry point (bsp_spmm), within the tolerance the other
SpMM tests use (1e-5 of the summation scale against FP64 for FP32 B, 1e-4
for BF16 B on the tensor cores), with FP32 B on the CUDA cores and with BF16
B on the tensor cores in the two shapes where the array also holds the tiled
copy of B and the split-K partials; and it checks that a problem whose
prototype sums exceed the array is refused.  It lives in its own file,
collected last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _p(t):
    return C.c_void_p(t.data_ptr())


def _noalloc(words, M, K, B, Cout, plan):
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    dt = capi.BF16 if B.dtype == torch.bfloat16 else capi.F32
    return capi.lib().bsp_spmm_noalloc(_p(words), M, K, _p(B), dt, B.stride(0), B.shape[1],
                                       _p(Cout), Cout.stride(0), plan.handle, stream)


def test_noalloc_matches_workspace_entry_point_twice():
    M, K, N = 2048, 4096, 512
    A, _, _ = W.clustered_bits(M, K, n_proto=16, p_proto=0.05, p_flip=0.003, seed_proto=31,
                               seed_rows=32)
    words = W.pack_bits(A)
    wd = torch.from_numpy(words.view(np.int32)).cuda()
    plan = ops.Plan(wd, K, mode=capi.PLAN_PROTO)
    assert plan.info()["mode"] == capi.PLAN_PROTO and plan.workspace_bytes(N) > 0
    C64 = Cabs = None
    for call, seed in enumerate((33, 34)):
        Bn = np.random.default_rng(seed).standard_normal((K, N)).astype(np.float32)
        B = torch.from_numpy(Bn).cuda()
        ref = ops.spmm(wd, K, B, plan=plan)                    # workspace entry point
        out = torch.full((M, N), float("nan"), device="cuda")
        assert _noalloc(wd, M, K, B, out, plan) == capi.BSP_OK
        torch.cuda.synchronize()
        assert capi.device_status() == 0
        C64 = O.spmm_f64(words, K, Bn)
        Cabs = O.spmm_abs_f64(words, K, Bn)
        scale = np.where(Cabs > 0, Cabs, 1.0)
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all(), call
        assert (np.abs(got - want) / scale).max() <= TOL, call
        assert (np.abs(got.astype(np.float64) - C64) / scale).max() <= TOL, call


@pytest.mark.parametrize("M", [8192, 512])
def test_noalloc_bf16_tensor_cores_twice(M, monkeypatch):
    """BF16 B on the tensor cores: with 8192 rows (32 row blocks) the tiled
    copy of B goes into the array; with 512 rows (two output tiles) the
    split-K partials do.  Two calls in a row with different B, each against
    bsp_spmm and FP64."""
    monkeypatch.setenv("BSP_TC", "1")
    K, N = 4096, 256
    A, _, _ = W.clustered_bits(M, K, n_proto=8, p_proto=0.05, p_flip=0.003, seed_proto=M, seed_rows=M + 1)
    words = W.pack_bits(A)
    wd = torch.from_numpy(words.view(np.int32)).cuda()
    plan = ops.Plan(wd, K, mode=capi.PLAN_PROTO)
    for call, seed in enumerate((41, 42)):
        Bn = np.random.default_rng(seed + M).standard_normal((K, N)).astype(np.float32)
        b16 = W.f32_to_bf16_bits(Bn)
        Bx = W.bf16_bits_to_f32(b16)
        B = torch.from_numpy(b16.view(np.int16)).cuda().view(torch.bfloat16)
        ref = ops.spmm(wd, K, B, plan=plan)
        out = torch.full((M, N), float("nan"), device="cuda")
        assert _noalloc(wd, M, K, B, out, plan) == capi.BSP_OK
        torch.cuda.synchronize()
        assert capi.device_status() == 0
        scale = np.where(O.spmm_abs_f64(words, K, Bx) > 0, O.spmm_abs_f64(words, K, Bx), 1.0)
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all(), call
        assert (np.abs(got - want) / scale).max() <= 1e-4, call
        assert (np.abs(got.astype(np.float64) - O.spmm_f64(words, K, Bx)) / scale).max() <= 1e-4, call


def test_noalloc_rejects_prototype_sums_beyond_its_array():
    M, K = 1024, 2048
    A, _, _ = W.clustered_bits(M, K, n_proto=64, p_proto=0.05, p_flip=0.002, seed_proto=35,
                               seed_rows=36)
    wd = torch.from_numpy(W.pack_bits(A).view(np.int32)).cuda()
    plan = ops.Plan(wd, K, mode=capi.PLAN_PROTO)
    n_proto = plan.info()["n_proto"]
    N = ((8 << 20) // (4 * max(n_proto, 1)) + 64) // 8 * 8   # prototype sums just past 8 MiB
    assert plan.workspace_bytes(N, preferred=False) > (8 << 20)
    B = torch.zeros((K, N), device="cuda")
    out = torch.zeros((M, N), device="cuda")
    assert _noalloc(wd, M, K, B, out, plan) == -8  # BSP_ERR_CAPACITY, refused before any launch
