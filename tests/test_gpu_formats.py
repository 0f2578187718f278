"""Interchange formats on the GPU against the oracle: 8x8 bitmap tiles
(source/src/main.cu:692-779) and tiled CSR (main.cu:499-588)."""
import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import dev, words_dev, words_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,K,p", [(37, 45, 0.1), (1024, 1024, 0.01), (8, 8, 1.0), (1000, 33, 0.3),
                                   (4096, 4096, 0.0005), (5, 300, 0.0)])
def test_rows_to_tiles8_and_back(M, K, p):
    A = np.random.default_rng(M + K).random((M, K)) < p
    w = W.pack_bits(A)
    bmp, tr, tc, off = ops.rows_to_tiles8(words_dev(w), K)
    obmp, otr, otc, ooff = O.rows_to_tiles8(w, M, K)
    assert np.array_equal(bmp.cpu().numpy().view(np.uint64), obmp)
    assert np.array_equal(tr.cpu().numpy(), otr)
    assert np.array_equal(tc.cpu().numpy(), otc)
    assert np.array_equal(off.cpu().numpy(), ooff)
    back = ops.tiles8_to_rows(bmp, tr, tc, M, K)
    assert np.array_equal(words_host(back), w)


def test_tiles8_to_rows_any_order_and_outside_tiles():
    A = np.random.default_rng(9).random((60, 70)) < 0.2
    w = W.pack_bits(A)
    bmp, tr, tc, _ = O.rows_to_tiles8(w, 60, 70)
    perm = np.random.default_rng(1).permutation(len(bmp))
    # an extra tile outside the matrix is ignored
    bmp2 = np.concatenate([bmp[perm], np.array([0xffffffffffffffff], np.uint64)])
    tr2 = np.concatenate([tr[perm], np.array([100], np.int32)])
    tc2 = np.concatenate([tc[perm], np.array([0], np.int32)])
    back = ops.tiles8_to_rows(dev(bmp2.view(np.int64)), dev(tr2), dev(tc2), 60, 70)
    assert np.array_equal(words_host(back), w)


def _random_csr(rng, M, K, p, shuffle=False):
    A = rng.random((M, K)) < p
    row_ptr = np.concatenate([[0], np.cumsum(A.sum(1))]).astype(np.int32)
    cols = [np.nonzero(A[i])[0] for i in range(M)]
    if shuffle:
        cols = [rng.permutation(c) for c in cols]
    col = np.concatenate(cols).astype(np.int32)
    val = rng.standard_normal(len(col)).astype(np.float32)
    return row_ptr, col, val


@pytest.mark.parametrize("M,K,TR,TC,p,shuffle", [(100, 70, 16, 32, 0.05, False), (37, 300, 8, 64, 0.1, True),
                                                 (2048, 2048, 512, 2048, 0.01, False),
                                                 (300, 5000, 7, 100, 0.02, True), (64, 64, 64, 64, 0.9, False)])
def test_csr_to_tiled_matches_oracle(M, K, TR, TC, p, shuffle):
    rng = np.random.default_rng(M * 3 + K)
    rp, col, val = _random_csr(rng, M, K, p, shuffle)
    acc, toff, tcol, tval = ops.csr_to_tiled(dev(rp), dev(col), M, K, TR, TC, values=dev(val))
    oacc, otoff, otcol, otval = O.csr_to_tiled(rp, col, val, M, K, TR, TC)
    assert np.array_equal(acc.cpu().numpy(), oacc)
    assert np.array_equal(toff.cpu().numpy(), otoff)
    assert np.array_equal(tcol.cpu().numpy(), otcol)
    assert np.array_equal(tval.cpu().numpy(), otval)
    # without values, and with 1-byte values (the reference's int8 value type)
    acc2, _, tcol2, none = ops.csr_to_tiled(dev(rp), dev(col), M, K, TR, TC)
    assert none is None and np.array_equal(tcol2.cpu().numpy(), otcol)
    v8 = (np.arange(len(col)) % 251 - 125).astype(np.int8)
    _, _, _, tv8 = ops.csr_to_tiled(dev(rp), dev(col), M, K, TR, TC, values=dev(v8))
    _, _, _, ov = O.csr_to_tiled(rp, col, v8.astype(np.float32), M, K, TR, TC)
    assert np.array_equal(tv8.cpu().numpy().astype(np.float32), ov)
