"""The oracle's output-side and interchange-format restatements against the
reference's own outputs, frozen in tests/golden/reference_small.npz by
gen_golden.py from the reference code built into oracle/_ref/:

* csr2tiledcsr (source/src/main.cu:499-588), three tile shapes;
* pre_spgemm (source/src/transform.cuh:984-1157): the symbolic output mask
  and the first-fit grouping of the output rows;
* coo2bmp_noTuple_d with find_tile_index / absolute2relative /
  bmp_popcount_d (main.cu:692-779, mm.h:83-144): 8x8 bitmap tiles;
* the 1024x1024 Bernoulli(0.1) matrix of the small plain SpMM: packing
  (main.cu:591-628) and row groups (main.cu:50-247) at the reference's own
  512-row tiles.

When the reference checkout is present the live reference code is also run
on fresh inputs."""
import numpy as np
import pytest

import oracle as O
from bitwise_spgemm_gb300 import workloads as W

C2T = ("256x256", "64x64", "32x128")
PRE = ("256", "64")
BMP = ("64x64", "37x91", "200x130")


@pytest.mark.parametrize("name", C2T)
def test_csr_to_tiled_matches_csr2tiledcsr_output(golden, name):
    M, K, th, tw = (int(x) for x in golden["c2t_%s_shape" % name])
    acc, toff, tcol, tval = O.csr_to_tiled(golden["c2t_%s_row_ptr" % name], golden["c2t_%s_col" % name],
                                           golden["c2t_%s_val" % name], M, K, th, tw)
    assert np.array_equal(acc, golden["c2t_%s_tile_nnz_acc" % name])
    assert np.array_equal(toff, golden["c2t_%s_tiled_offset" % name])
    assert np.array_equal(tcol, golden["c2t_%s_tiled_col" % name])
    assert np.array_equal(tval.view(np.uint32), golden["c2t_%s_tiled_val" % name].view(np.uint32))
    # the per-(row, tile column) counts the reference keeps are the row-pointer differences
    trn = golden["c2t_%s_tile_row_nnz" % name]
    Kt = K // tw
    for t in range(toff.shape[0]):
        ty, tx = divmod(t, Kt)
        assert np.array_equal(np.diff(toff[t]), trn[ty * th:(ty + 1) * th, tx])


@pytest.mark.parametrize("name", PRE)
def test_symbolic_mask_and_output_groups_match_pre_spgemm(golden, name):
    M, K, N, t = (int(x) for x in golden["pre_%s_shape" % name])
    a = golden["pre_%s_A_words" % name]
    b = golden["pre_%s_B_words_msb" % name]
    sym = O.symbolic_rows(a, K, b, N)
    assert np.array_equal(sym, golden["pre_%s_c_bits" % name])
    g = O.group_rows(sym, t, 2)
    gid = golden["pre_%s_group_idx" % name]
    assert (gid == -1).any() and (gid == 1).any()  # the case exercises spills and group 1
    assert np.array_equal(g["group_id"], gid)
    assert np.array_equal(g["group_mask"], golden["pre_%s_group_mask" % name])
    assert int(g["grouped_nnz"][0]) == int(golden["pre_%s_nnz" % name][0])


@pytest.mark.parametrize("name", BMP)
def test_rows_to_tiles8_matches_coo2bmp(golden, name):
    M, K = (int(x) for x in golden["bmp_%s_shape" % name])
    bmp, tr, tc, off = O.rows_to_tiles8(golden["bmp_%s_words" % name], M, K)
    assert np.array_equal(bmp, golden["bmp_%s_bmp" % name])
    assert np.array_equal(tr, golden["bmp_%s_tile_row" % name])
    assert np.array_equal(tc, golden["bmp_%s_tile_col" % name])
    assert np.array_equal(off[:-1].astype(np.uint32), golden["bmp_%s_idx" % name])
    assert int(off[-1]) == int(W.unpack_bits(golden["bmp_%s_words" % name], K).sum())


def test_small_plain_matrix_packing_and_groups(golden):
    c1 = W.config1()
    A = W.unpack_bits(c1["words"], c1["K"]).astype(np.float32)
    assert np.array_equal(O.pack_rows(A, msb_first=True), golden["c1_words_msb"])
    g = O.group_rows(golden["c1_words_msb"], 512, 2)
    ref = golden["c1_group_id_ref"]
    # spilled rows carry MAX_GROUP_NUM (= 2) in the reference (main.cu:184); the intent is -1
    assert np.array_equal(np.where(ref == 2, -1, ref), g["group_id"])
    assert np.array_equal(g["group_mask"], golden["c1_group_mask_ref"])
    assert int(g["grouped_nnz"][0]) == int(golden["c1_group_nnz_ref"][0])


def _live():
    from oracle import ref as R
    if not R.build_ref.available():
        pytest.skip("reference checkout not present")
    return R


@pytest.mark.parametrize("seed", [1, 2])
def test_live_reference_output_side(seed):
    R = _live()
    rng = np.random.default_rng(seed)
    M, K, N, t = 512, 256, 160, 256
    A = rng.random((M, K)) < 0.03
    Bd = (rng.random((K, N)) < 0.04).astype(np.float32)
    bw = R.dense2bitmask(Bd, 64)
    rp = np.concatenate([[0], np.cumsum(A.sum(1))]).astype(np.int32)
    col = np.nonzero(A)[1].astype(np.int32)
    val = rng.standard_normal(len(col)).astype(np.float32)
    tl = R.csr2tiledcsr(rp, col, val, M, K, t, t)
    acc, toff, tcol, tval = O.csr_to_tiled(rp, col, val, M, K, t, t)
    assert np.array_equal(acc, tl["tile_nnz_acc"]) and np.array_equal(toff, tl["tiled_offset"])
    assert np.array_equal(tcol, tl["tiled_col"]) and np.array_equal(tval, tl["tiled_val"])
    o = R.pre_spgemm(bw, tl, M, K, N, t)
    sym = O.symbolic_rows(W.pack_bits(A), K, bw, N)
    assert np.array_equal(sym, o["c_bits"])
    g = O.group_rows(sym, t, 2)
    assert np.array_equal(g["group_id"], o["group_idx"])
    assert np.array_equal(g["group_mask"], o["group_mask"])
    M2, K2 = 123, 77
    A2 = rng.random((M2, K2)) < 0.1
    r, c = np.nonzero(A2)
    perm = rng.permutation(len(r))
    bmp, tr, tc, ix, _ = R.coo2bmp(r[perm], c[perm], np.ones(len(r), np.float32), M2, K2)
    obmp, otr, otc, ooff = O.rows_to_tiles8(W.pack_bits(A2), M2, K2)
    assert np.array_equal(bmp, obmp) and np.array_equal(tr, otr) and np.array_equal(tc, otc)
    assert np.array_equal(ix, ooff[:-1].astype(np.uint32))
