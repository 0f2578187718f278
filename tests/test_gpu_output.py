"""Output side and multi-bit operands on the GPU: symbolic output masks and
their first-fit grouping, bit-plane products and the int8 path, against the
oracle (source/src/transform.cuh:1028-1157 and :2199-2246, main.cu:895-910)."""
import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import dev, words_dev, words_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,K,N,pa,pb", [(300, 70, 90, 0.05, 0.1), (64, 4096, 5000, 0.002, 0.01),
                                         (1000, 33, 31, 0.2, 0.05), (5, 32, 8192, 0.5, 0.001),
                                         (128, 256, 1, 0.1, 0.5)])
def test_symbolic_rows_match_oracle(M, K, N, pa, pb):
    rng = np.random.default_rng(M * 7 + N)
    A = rng.random((M, K)) < pa
    A[M // 2] = False  # an empty row
    Bm = rng.random((K, N)) < pb
    a, b = W.pack_bits(A), W.pack_bits(Bm)
    got = words_host(ops.symbolic_rows(words_dev(a), K, words_dev(b), N))
    assert np.array_equal(got, O.symbolic_rows(a, K, b, N))
    # the mask is the nonzero pattern of the integer product
    prod = (A.astype(np.int64) @ Bm.astype(np.int64)) > 0
    assert np.array_equal(got, W.pack_bits(prod))


@pytest.mark.parametrize("N,pb", [(31, 0.05), (2056, 0.01), (8192, 0.002), (300, 0.3)])
def test_symbolic_rows_through_plan(N, pb):
    """Clustered A (plus rows that fit no cluster): the planned pass — the
    clusters' bit-sliced counts, then each row's added and removed columns —
    gives the same masks as the direct OR walk and the oracle, including
    dense B masks where counts run high and removed columns matter."""
    from bitwise_spgemm_gb300 import capi
    rng = np.random.default_rng(N)
    A, _, _ = W.clustered_bits(1500, 2500, n_proto=7, p_proto=0.08, p_flip=0.006, seed_proto=N, seed_rows=N + 1)
    A[::13] = rng.random((A[::13].shape[0], 2500)) < 0.03  # rows that fit no cluster
    A[5] = False                                             # an empty row
    Bm = rng.random((2500, N)) < pb
    a, b = W.pack_bits(A), W.pack_bits(Bm)
    ad, bd = words_dev(a), words_dev(b)
    plan = ops.Plan(ad, 2500, mode=capi.PLAN_PROTO)
    info = plan.info()
    assert info["mode"] == capi.PLAN_PROTO and info["direct_rows"] > 0 and info["delta_nnz"] > 0
    got = words_host(ops.symbolic_rows(ad, 2500, bd, N, plan=plan))
    assert np.array_equal(got, words_host(ops.symbolic_rows(ad, 2500, bd, N)))
    assert np.array_equal(got, O.symbolic_rows(a, 2500, b, N))
    assert capi.device_status() == 0


@pytest.mark.parametrize("TR,G", [(512, 2), (64, 4)])
def test_output_grouping_of_symbolic_masks(TR, G):
    # pre_spgemm's second half: first-fit grouping of the output rows
    rng = np.random.default_rng(TR + G)
    A = rng.random((1024, 256)) < 0.01
    Bm = rng.random((256, 512)) < 0.01
    a, b = W.pack_bits(A), W.pack_bits(Bm)
    cw = ops.symbolic_rows(words_dev(a), 256, words_dev(b), 512)
    g = ops.group_rows(cw, TR, G)
    o = O.group_rows(O.symbolic_rows(a, 256, b, 512), TR, G)
    for k in ("group_id", "group_row", "spill_cnt", "spill_nnz", "spill_rows"):
        assert np.array_equal(g[k].cpu().numpy(), o[k]), k
    assert np.array_equal(words_host(g["group_mask"]), o["group_mask"])


def _int8(rng, M, K):
    A = rng.integers(-128, 128, (M, K), dtype=np.int16).astype(np.int8)
    A[0, : min(K, 4)] = [-128, 127, -1, 0][: min(K, 4)]
    return A


@pytest.mark.parametrize("M,K,N", [(200, 300, 256), (64, 1000, 96), (33, 65, 40), (8, 4096, 512)])
def test_spmm_i8_integer_B_is_exact(M, K, N):
    rng = np.random.default_rng(K)
    A = _int8(rng, M, K)
    B = rng.integers(-8, 9, (K, N)).astype(np.float32)
    C = ops.spmm_i8(dev(A), dev(B)).cpu().numpy()
    assert np.array_equal(C.astype(np.float64), A.astype(np.float64) @ B.astype(np.float64))


@pytest.mark.parametrize("kind", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("M,K,N", [(128, 512, 128), (50, 77, 24), (17, 300, 33)])
def test_bitplane_spmm_matches_oracle(kind, M, K, N):
    rng = np.random.default_rng(M + K + N)
    A = _int8(rng, M, K)
    Bf = rng.standard_normal((K, N), dtype=np.float32)
    tdt = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[kind]
    Bt = dev(Bf).to(tdt)
    Bq = Bt.float().cpu().numpy()  # the values the kernel reads
    planes = ops.bitplanes(dev(A.view(np.uint8)), 8)
    C = ops.bitplane_spmm(planes, K, Bt).cpu().numpy()
    C64 = O.bitplane_spmm_f64(A, Bq)
    Cabs = np.abs(A.astype(np.float64)) @ np.abs(Bq.astype(np.float64))
    ms, _, mn = O.rel_errors(C, C64, Cabs)
    assert ms <= 1e-5 and mn <= 1e-5, (ms, mn)
    # the int8 entry point computes the same thing
    C2 = ops.spmm_i8(dev(A), Bt).cpu().numpy()
    assert np.array_equal(C, C2)


def test_unsigned_planes_and_fewer_planes():
    rng = np.random.default_rng(3)
    U = rng.integers(0, 256, (96, 200), dtype=np.int16).astype(np.uint8)
    B = rng.integers(-4, 5, (200, 64)).astype(np.float32)
    planes = ops.bitplanes(dev(U), 8)
    C = ops.bitplane_spmm(planes, 200, dev(B), signed=False).cpu().numpy()
    assert np.array_equal(C.astype(np.float64), U.astype(np.float64) @ B.astype(np.float64))
    # the low 3 planes only: values mod 8
    C3 = ops.bitplane_spmm(planes[:3].contiguous(), 200, dev(B), signed=False).cpu().numpy()
    assert np.array_equal(C3.astype(np.float64), (U % 8).astype(np.float64) @ B.astype(np.float64))


@pytest.mark.parametrize("kind", ["bf16", "f16", "f32"])
@pytest.mark.parametrize("M,K,N,d", [(512, 1024, 256, 0.05), (100, 77, 40, 0.3), (1024, 4096, 512, 0.02)])
def test_int8_planes_along_k(kind, M, K, N, d, monkeypatch):
    # C = [P_0 | ... | P_7] · [w_0 B; ...; w_7 B] through the planned bitmap
    # SpMM, on the tensor cores (BSP_TC=1) and on the CUDA cores (BSP_TC=0)
    rng = np.random.default_rng(M + K + N)
    A = np.where(rng.random((M, K)) < d, rng.integers(-128, 128, (M, K)), 0).astype(np.int8)
    A[0, :3] = [-128, 127, -1]
    Bf = rng.standard_normal((K, N), dtype=np.float32)
    tdt = {"f32": torch.float32, "bf16": torch.bfloat16, "f16": torch.float16}[kind]
    Bt = dev(Bf).to(tdt)
    Bq = Bt.float().cpu().numpy()
    C64 = O.bitplane_spmm_f64(A, Bq)
    # error scale of this form: sum_b |w_b| (P_b |B|) — the weighted plane
    # terms it adds (an int8 -1 sets all 8 planes, |weights| summing to 255)
    U = A.view(np.uint8)
    W8 = sum((2.0 ** b) * ((U >> b) & 1).astype(np.float64) for b in range(8))
    Cabs = W8 @ np.abs(Bq.astype(np.float64))
    # the stacked B is exact: block b row k = w_b * B[k]
    Bs = ops.stack_planes_b(Bt, K).float().cpu().numpy()
    Kp = ((K + 31) // 32) * 32
    for b, w in enumerate([1, 2, 4, 8, 16, 32, 64, -128]):
        assert np.array_equal(Bs[b * Kp: b * Kp + K], w * Bq)
        assert not Bs[b * Kp + K: (b + 1) * Kp].any()
    # the plane rows hold the same bits as the plane-major layout
    pr = ops.bitplanes_rows(dev(U)).cpu().numpy().view(np.uint32)
    pm = O.bitplanes(U, 8)
    assert np.array_equal(pr.reshape(M, 8, -1).transpose(1, 0, 2), pm)
    tol = 1e-5 if kind == "f32" else 1e-3
    for tc in ("1", "0"):
        if kind == "f32" and tc == "1":
            continue
        monkeypatch.setenv("BSP_TC", tc)
        mat = ops.Int8Matrix(dev(A))
        C = mat.matmul(Bt).cpu().numpy()
        mat.close()
        ms, _, mn = O.rel_errors(C, C64, Cabs)
        assert ms <= tol, (tc, ms, mn)
