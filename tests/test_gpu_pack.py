"""Packing kernels on the GPU against the oracle and the reference fixtures."""
import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import dev, words_host

pytestmark = pytest.mark.gpu


def test_pack_rows_reference_fixture(golden):
    d = golden["pack_dense"]
    got = words_host(ops.pack_rows(dev(d), bit_order=capi.MSB_FIRST))
    assert np.array_equal(got, golden["pack_words_msb"])
    got_lsb = words_host(ops.pack_rows(dev(d)))
    assert np.array_equal(got_lsb, O.pack_rows(d))


@pytest.mark.parametrize("dt", [torch.float32, torch.float16, torch.bfloat16, torch.int8, torch.uint8])
@pytest.mark.parametrize("shape", [(1, 1), (37, 45), (64, 1024), (129, 97), (300, 4100)])
def test_pack_rows_dtypes_shapes(dt, shape):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    M, K = shape
    bits = rng.random((M, K)) < 0.2
    vals = np.where(bits, rng.integers(1, 100, (M, K)), 0).astype(np.float32)
    t = torch.from_numpy(vals).to(dt).cuda()
    ref = W.pack_bits(bits)
    for order in (capi.LSB_FIRST, capi.MSB_FIRST):
        got = words_host(ops.pack_rows(t, bit_order=order))
        exp = O.pack_rows(bits.astype(np.uint8), msb_first=order == capi.MSB_FIRST)
        assert np.array_equal(got, exp)
    assert np.array_equal(words_host(ops.pack_rows(t)), ref)


def test_pack_rows_strided_and_special_values():
    rng = np.random.default_rng(1)
    base = rng.standard_normal((50, 200)).astype(np.float32)
    base[base < 0.5] = 0.0
    base[0, :8] = [-0.0, np.nan, np.inf, -np.inf, 1e-42, 0.0, -1e-42, 0.0]
    t = torch.from_numpy(base).cuda()[:, 10:150]  # ld = 200, K = 140
    got = words_host(ops.pack_rows(t))
    assert np.array_equal(got, O.pack_rows(np.ascontiguousarray(base[:, 10:150])))


@pytest.mark.parametrize("shape", [(1, 1), (37, 45), (64, 1024), (300, 97)])
def test_pack_cols_and_transpose(shape):
    rng = np.random.default_rng(sum(shape))
    M, K = shape
    bits = rng.random((M, K)) < 0.3
    t = torch.from_numpy(bits.astype(np.float32)).cuda()
    exp = O.pack_cols(bits.astype(np.uint8))
    assert np.array_equal(words_host(ops.pack_cols(t)), exp)
    words = ops.pack_rows(t)
    assert np.array_equal(words_host(ops.transpose_bits(words, M, K)), exp)
    back = ops.unpack_rows(words, M, K)
    assert torch.equal(back.cpu(), t.cpu())
    for dt in (torch.bfloat16, torch.float16, torch.uint8):
        assert torch.equal(ops.unpack_rows(words, M, K, dtype=dt).float().cpu(), t.cpu())


def test_bitplanes_reference_fixture(golden):
    v = golden["planes_u8"]
    got = ops.bitplanes(dev(v)).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, O.bitplanes(v))
    ref = golden["planes_ref"]
    assert np.array_equal(got, W.pack_bits(ref.reshape(-1, v.shape[1]).astype(bool)).reshape(got.shape))


def test_bitplanes_ragged():
    rng = np.random.default_rng(9)
    v = rng.integers(0, 256, (33, 70)).astype(np.uint8)
    for planes in (1, 3, 8):
        got = ops.bitplanes(dev(v), planes=planes).cpu().numpy().view(np.uint32)
        assert np.array_equal(got, O.bitplanes(v, planes))


@pytest.mark.parametrize("M,K,LD", [(64, 4096, 4096), (17, 1000, 1040), (5, 16, 16), (300, 512, 528),
                                    (2, 530, 544)])
def test_bitplanes_vector_path(M, K, LD):
    # 16-byte aligned rows take the vector kernel (ragged row ends included)
    rng = np.random.default_rng(M + K)
    full = rng.integers(0, 256, (M, LD)).astype(np.uint8)
    t = dev(full)[:, :K]
    v = full[:, :K]
    for planes, order in ((8, capi.LSB_FIRST), (3, capi.LSB_FIRST), (8, capi.MSB_FIRST)):
        got = ops.bitplanes(t, planes=planes, bit_order=order).cpu().numpy().view(np.uint32)
        assert np.array_equal(got, O.bitplanes(np.ascontiguousarray(v), planes, msb_first=order == capi.MSB_FIRST))
