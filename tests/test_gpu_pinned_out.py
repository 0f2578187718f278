"""The CUDA library against the reference's own outputs (frozen in
tests/golden/reference_small.npz) for the output side and the interchange
formats: csr2tiledcsr (source/src/main.cu:499-588), pre_spgemm's symbolic
mask and output grouping (source/src/transform.cuh:984-1157), coo2bmp's 8x8
bitmap tiles (main.cu:692-779, mm.h:83-144), and packing plus row groups of
the 1024x1024 Bernoulli(0.1) matrix of the small plain SpMM (main.cu:591-628,
:50-247)."""
import numpy as np
import pytest

from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import dev, words_dev, words_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["256x256", "64x64", "32x128"])
def test_csr_to_tiled_matches_csr2tiledcsr(golden, name):
    M, K, th, tw = (int(x) for x in golden["c2t_%s_shape" % name])
    rp, col, val = (golden["c2t_%s_%s" % (name, k)] for k in ("row_ptr", "col", "val"))
    acc, toff, tcol, tval = ops.csr_to_tiled(dev(rp), dev(col), M, K, th, tw, values=dev(val))
    assert np.array_equal(acc.cpu().numpy(), golden["c2t_%s_tile_nnz_acc" % name])
    assert np.array_equal(toff.cpu().numpy(), golden["c2t_%s_tiled_offset" % name])
    assert np.array_equal(tcol.cpu().numpy(), golden["c2t_%s_tiled_col" % name])
    assert np.array_equal(tval.cpu().numpy().view(np.uint32), golden["c2t_%s_tiled_val" % name].view(np.uint32))


@pytest.mark.parametrize("name", ["256", "64"])
@pytest.mark.parametrize("planned", [False, True])
def test_symbolic_mask_and_output_groups_match_pre_spgemm(golden, name, planned):
    M, K, N, t = (int(x) for x in golden["pre_%s_shape" % name])
    a = golden["pre_%s_A_words" % name]
    b = golden["pre_%s_B_words_msb" % name]
    ad = words_dev(a)
    plan = ops.Plan(ad, K, mode=capi.PLAN_PROTO) if planned else None
    sym = ops.symbolic_rows(ad, K, words_dev(b), N, plan=plan)
    assert np.array_equal(words_host(sym), golden["pre_%s_c_bits" % name])
    g = ops.group_rows(sym, t, 2)
    assert np.array_equal(g["group_id"].cpu().numpy(), golden["pre_%s_group_idx" % name])
    assert np.array_equal(words_host(g["group_mask"]), golden["pre_%s_group_mask" % name])
    assert int(g["grouped_nnz"].item()) == int(golden["pre_%s_nnz" % name][0])
    if plan is not None:
        plan.close()
    assert capi.device_status() == 0


@pytest.mark.parametrize("name", ["64x64", "37x91", "200x130"])
def test_rows_to_tiles8_matches_coo2bmp(golden, name):
    M, K = (int(x) for x in golden["bmp_%s_shape" % name])
    w = golden["bmp_%s_words" % name]
    bmp, tr, tc, off = ops.rows_to_tiles8(words_dev(w), K)
    assert np.array_equal(bmp.cpu().numpy().view(np.uint64), golden["bmp_%s_bmp" % name])
    assert np.array_equal(tr.cpu().numpy(), golden["bmp_%s_tile_row" % name])
    assert np.array_equal(tc.cpu().numpy(), golden["bmp_%s_tile_col" % name])
    assert np.array_equal(off.cpu().numpy()[:-1].astype(np.uint32), golden["bmp_%s_idx" % name])


def test_small_plain_matrix_packing_and_groups(golden):
    c1 = W.config1()
    A = W.unpack_bits(c1["words"], c1["K"]).astype(np.float32)
    w = ops.pack_rows(dev(A), bit_order=capi.MSB_FIRST)
    assert np.array_equal(words_host(w), golden["c1_words_msb"])
    assert np.array_equal(words_host(ops.pack_rows(dev(A))), c1["words"])
    g = ops.group_rows(w, 512, 2)
    ref = golden["c1_group_id_ref"]
    assert np.array_equal(g["group_id"].cpu().numpy(), np.where(ref == 2, -1, ref))
    assert np.array_equal(words_host(g["group_mask"]), golden["c1_group_mask_ref"])
    assert int(g["grouped_nnz"].item()) == int(golden["c1_group_nnz_ref"][0])
