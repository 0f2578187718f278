"""First-fit grouping on the GPU: reference fixture and oracle parity."""
import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import words_dev, words_host

pytestmark = pytest.mark.gpu


def _cmp(words, tr, G):
    g = ops.group_rows(words_dev(words), tr, G)
    o = O.group_rows(words, tr, G)
    for k in ("group_id", "group_row", "spill_cnt", "spill_nnz", "spill_rows"):
        assert np.array_equal(g[k].cpu().numpy(), o[k]), k
    assert np.array_equal(words_host(g["group_mask"]), o["group_mask"])
    assert int(g["grouped_nnz"].item()) == int(o["grouped_nnz"][0])
    return g


def test_group_rows_reference_fixture(golden):
    TR = int(golden["group_tile_rows"])
    w = golden["group_words_msb"]
    g = _cmp(w, TR, 2)
    ref = golden["group_id_ref"]
    assert np.array_equal(np.where(ref == 2, -1, ref), g["group_id"].cpu().numpy())
    assert np.array_equal(words_host(g["group_mask"]), golden["group_mask_ref"])


@pytest.mark.parametrize("M,K,TR,G,p", [(1024, 1024, 512, 2, 0.1), (1000, 100, 64, 4, 0.05),
                                        (77, 33, 7, 1, 0.3), (2048, 256, 2048, 32, 0.02),
                                        (1, 32, 4096, 2, 0.5)])
def test_group_rows_random(M, K, TR, G, p):
    rng = np.random.default_rng(M + K)
    words = W.pack_bits(rng.random((M, K)) < p)
    _cmp(words, TR, G)


def test_group_to_dense_fixture(golden):
    TR = int(golden["group_tile_rows"])
    w_msb = golden["group_words_msb"]
    M, Kw = w_msb.shape
    w_lsb = np.array([int(f"{x:032b}"[::-1], 2) for x in w_msb.ravel()], np.uint32).reshape(w_msb.shape)
    g = O.group_rows(w_msb, TR, 2)
    vals = torch.from_numpy(np.ascontiguousarray(golden["g2d_values"])).cuda()
    out = ops.group_to_dense(vals, torch.from_numpy(g["group_id"]).cuda(), words_dev(w_lsb), M,
                             Kw * 32, TR, 2)
    assert np.array_equal(out.cpu().numpy(), golden["g2d_dense_ref"])
