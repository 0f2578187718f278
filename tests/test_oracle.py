"""The oracle against the reference: frozen golden outputs of the reference's
own kernels (tests/golden/reference_small.npz, made by gen_golden.py) and, when
the reference checkout is present, the live reference code built into
oracle/_ref/."""
import numpy as np
import pytest

import oracle as O
from bitwise_spgemm_gb300 import workloads as W


def test_pack_rows_matches_dense2bitmask(golden):
    d = golden["pack_dense"]
    assert np.array_equal(O.pack_rows(d, msb_first=True), golden["pack_words_msb"])
    lsb = O.pack_rows(d)
    brev = np.array([int(f"{x:032b}"[::-1], 2) for x in golden["pack_words_msb"].ravel()],
                    np.uint32).reshape(lsb.shape)
    assert np.array_equal(lsb, brev)
    # -0.0 is zero, NaN / inf / denormals are nonzero
    bits = W.unpack_bits(lsb, d.shape[1])
    assert np.array_equal(bits, (d != 0) | np.isnan(d))


def test_group_rows_matches_generate_groups_large(golden):
    TR = int(golden["group_tile_rows"])
    w = golden["group_words_msb"]
    g = O.group_rows(w, TR, 2)
    ref_gid = golden["group_id_ref"]
    # the reference stores MAX_GROUP_NUM (=2) for spilled rows (main.cu:184); intent is -1
    assert np.array_equal(np.where(ref_gid == 2, -1, ref_gid), g["group_id"])
    assert np.array_equal(golden["group_mask_ref"], g["group_mask"])
    assert int(golden["group_nnz_ref"][0]) == int(g["grouped_nnz"][0])
    # group values: value of the owning row at each column (MSB bit 31-i <-> column i)
    dense = golden["group_dense"]
    Kw = w.shape[1]
    gr = g["group_row"][:, :, ::-1]
    vals = np.zeros_like(golden["group_val_ref"])
    for t in range(gr.shape[0]):
        rb, ww = divmod(t, Kw)
        for gg in range(2):
            for i in range(32):
                r = gr[t, gg, i]
                if r >= 0:
                    vals[t, gg, i] = np.int8(dense[rb * TR + r, ww * 32 + i])
    assert np.array_equal(vals, golden["group_val_ref"])
    # spill bookkeeping is self-consistent
    spilled = (g["group_id"] == -1)
    assert spilled.sum() == g["spill_cnt"].sum() > 0


def test_group_to_dense_matches_group2dense(golden):
    TR = int(golden["group_tile_rows"])
    w_msb = golden["group_words_msb"]
    M, Kw = w_msb.shape
    K = Kw * 32
    g = O.group_rows(w_msb, TR, 2)
    # reference works on MSB-first bits; the oracle on LSB-first: reverse each
    # word and the 32-entry value vectors
    w_lsb = np.array([int(f"{x:032b}"[::-1], 2) for x in w_msb.ravel()], np.uint32).reshape(w_msb.shape)
    vals = golden["g2d_values"]
    # the reference reads value index i for column i (bit 31-i of its MSB word);
    # the oracle reads value index i for bit i of the LSB word, which is column i
    out = O.group_to_dense(np.ascontiguousarray(vals), g["group_id"], w_lsb, M, K, TR, 2)
    assert np.array_equal(out, golden["g2d_dense_ref"])


def test_bitplanes_match_uint8_layout_trans(golden):
    v = golden["planes_u8"]
    ref = golden["planes_ref"]  # [8][m][k] ints
    got = O.bitplanes(v, 8)
    m, k = v.shape
    assert np.array_equal(got, W.pack_bits(ref.reshape(8 * m, k).astype(bool)).reshape(8, m, -1))


def test_spmm_f32_is_bit_identical_to_reference_order(golden):
    A = golden["spmm_A01"].astype(bool)
    words = W.pack_bits(A)
    for bkey, ckey in (("spmm_B_int", "spmm_C_int_ref"), ("spmm_B_normal", "spmm_C_normal_ref")):
        C = O.spmm_f32(words, A.shape[1], golden[bkey])
        assert np.array_equal(C, golden[ckey]), bkey
    C64 = O.spmm_f64(words, A.shape[1], golden["spmm_B_int"])
    assert np.array_equal(C64.astype(np.float32), golden["spmm_C_int_ref"])


def test_bitserial_product(golden):
    A8 = golden["bitserial_A_u8"]
    B = golden["bitserial_B"]
    ref = golden["bitserial_C_ref"]
    # uint8 planes with weights 2^b (layout_trans.cu:165) == A(uint8) @ B exactly for small ints
    assert np.array_equal(ref.astype(np.float64), A8.astype(np.float64) @ B.astype(np.float64))
    # the int8 weighting of transform.cuh (-128 on plane 7) gives the signed product
    C = O.bitplane_spmm_f64(A8.view(np.int8), B)
    assert np.array_equal(C, A8.view(np.int8).astype(np.float64) @ B.astype(np.float64))


def test_check_verdicts(golden):
    A = golden["spmm_A01"].astype(np.float32)
    B = golden["spmm_B_normal"]
    assert bool(golden["check_good"]) and not bool(golden["check_bad"])
    assert O.check(A, B, golden["spmm_C_normal_ref"]) == -1
    assert O.check(A, B, golden["check_C_bad"]) == 3 * 64 + 5
    Cs = O.dense_check_sum(A, B)
    assert np.array_equal(Cs, golden["spmm_C_normal_ref"])
    assert np.array_equal(O.dense_check_sum(A, B, threads=4), Cs)


def test_oracle_edge_cases():
    rng = np.random.default_rng(3)
    # ragged K, M not a multiple of 32, empty rows
    M, K, N = 37, 45, 7
    bits = rng.random((M, K)) < 0.3
    bits[5] = False
    words = W.pack_bits(bits)
    assert words.shape == (M, 2)
    assert np.array_equal(O.pack_rows(bits.astype(np.float32)), words)
    assert np.array_equal(O.pack_rows(bits.astype(np.int8)), words)
    assert np.array_equal(O.unpack_rows(words, M, K), bits.astype(np.float32))
    B = rng.standard_normal((K, N)).astype(np.float32)
    C64 = O.spmm_f64(words, K, B)
    assert np.allclose(C64, bits.astype(np.float64) @ B.astype(np.float64), atol=1e-12)
    assert np.all(C64[5] == 0)
    t = O.transpose_bits(words, M, K)
    assert np.array_equal(t, W.pack_bits(bits.T))
    assert np.array_equal(O.pack_cols(bits.astype(np.float32)), t)
    G = rng.standard_normal((M, N)).astype(np.float32)
    dB = O.spmm_t_f64(words, M, K, G)
    assert np.allclose(dB, bits.T.astype(np.float64) @ G.astype(np.float64), atol=1e-12)
    X = B
    vals = O.sddmm_f64(words, M, K, G, X)
    full = G.astype(np.float64) @ X.astype(np.float64).T
    assert np.allclose(vals, full[bits], atol=1e-12)
    # empty matrix
    z = O.spmm_f64(np.zeros((0, 2), np.uint32), K, B)
    assert z.shape == (0, N)


def test_group_rows_edge_cases():
    rng = np.random.default_rng(4)
    words = (rng.integers(0, 2 ** 32, (50, 3), dtype=np.uint64) & rng.integers(0, 2 ** 32, (50, 3), dtype=np.uint64)).astype(np.uint32)
    words[::7] = 0
    for tr, mg in ((16, 1), (16, 2), (7, 4), (64, 32)):
        g = O.group_rows(words, tr, mg)
        Kw = words.shape[1]
        for t in range(g["group_mask"].shape[0]):
            rb, w = divmod(t, Kw)
            rows = words[rb * tr:(rb + 1) * tr, w]
            gid = g["group_id"][rb * tr:(rb + 1) * tr, w]
            for gg in range(mg):
                members = rows[gid == gg]
                acc = np.uint32(0)
                for m in members:
                    assert (acc & m) == 0
                    acc |= m
                assert acc == g["group_mask"][t, gg]
            assert (gid == -1).sum() == g["spill_cnt"][t]
            assert np.all(rows[gid == -1] != 0)


def test_symbolic_rows():
    rng = np.random.default_rng(5)
    A = rng.random((20, 70)) < 0.1
    Bm = rng.random((70, 90)) < 0.05
    c = O.symbolic_rows(W.pack_bits(A), 70, W.pack_bits(Bm), 90)
    assert np.array_equal(c, W.pack_bits((A.astype(int) @ Bm.astype(int)) > 0))


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(6).standard_normal(4096).astype(np.float32)
    x[:4] = [0.0, -0.0, 1e-40, 3.0e38]
    a = W.f32_to_bf16_bits(x)
    b = torch.from_numpy(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(a, b)


live = pytest.mark.skipif(not __import__("oracle.ref", fromlist=["x"]).build_ref.available(),
                          reason="reference checkout absent (fixtures cover this elsewhere)")


@live
def test_live_reference_random_cases():
    from oracle import ref as R
    rng = np.random.default_rng(11)
    for M, K, TR, p in ((128, 64, 32, 0.2), (256, 96, 128, 0.05), (64, 32, 64, 0.5)):
        bits = rng.random((M, K)) < p
        dense = np.where(bits, rng.integers(1, 50, (M, K)), 0).astype(np.float32)
        wr = R.dense2bitmask(dense, TR)
        assert np.array_equal(wr, O.pack_rows(dense, msb_first=True))
        gr = R.generate_groups_large(wr, dense, TR)
        go = O.group_rows(wr, TR, 2)
        assert np.array_equal(np.where(gr["group_id"] == 2, -1, gr["group_id"]), go["group_id"])
        assert np.array_equal(gr["group_mask"], go["group_mask"])
        A01 = bits[:16].astype(np.uint8)
        B = rng.standard_normal((K, 24)).astype(np.float32)
        Cr = R.uint8_spmm(R.uint8_layout_trans(A01), B)
        assert np.array_equal(Cr, O.spmm_f32(W.pack_bits(bits[:16]), K, B))
        assert R.check(A01.astype(np.float32), B, Cr)


def _tiles8_numpy(A):
    # find_tile_index (source/src/mm.h:83-104): tile = (r/8)*ncols8 + c/8,
    # position bit = (r%8)*8 + c%8; tiles OR-reduced in ascending tile index
    # and offsets = exclusive scan of popcounts (main.cu:692-779)
    M, K = A.shape
    ncols8 = (K + 7) // 8
    tiles = {}
    for r, c in zip(*np.nonzero(A)):
        t = (r // 8) * ncols8 + c // 8
        tiles[t] = tiles.get(t, 0) | (1 << int((r % 8) * 8 + c % 8))
    keys = sorted(tiles)
    bmp = np.array([tiles[t] for t in keys], np.uint64)
    pc = [bin(tiles[t]).count("1") for t in keys]
    off = np.concatenate([[0], np.cumsum(pc)]).astype(np.int32)
    return bmp, np.array([t // ncols8 for t in keys], np.int32), np.array([t % ncols8 for t in keys], np.int32), off


@pytest.mark.parametrize("M,K,p", [(37, 45, 0.1), (8, 8, 1.0), (64, 200, 0.02), (3, 5, 0.5)])
def test_tiles8_oracle_matches_reference_formulas(M, K, p):
    A = np.random.default_rng(M * K).random((M, K)) < p
    w = W.pack_bits(A)
    got = O.rows_to_tiles8(w, M, K)
    ref = _tiles8_numpy(A)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    assert np.array_equal(O.tiles8_to_rows(got[0], got[1], got[2], M, K), w)


def _random_csr(rng, M, K, p, shuffle=False):
    A = rng.random((M, K)) < p
    row_ptr = np.concatenate([[0], np.cumsum(A.sum(1))]).astype(np.int32)
    cols = [np.nonzero(A[i])[0] for i in range(M)]
    if shuffle:
        cols = [rng.permutation(c) for c in cols]
    col = np.concatenate(cols).astype(np.int32) if cols else np.zeros(0, np.int32)
    val = rng.standard_normal(len(col)).astype(np.float32)
    return row_ptr, col, val


@pytest.mark.parametrize("M,K,TR,TC,shuffle", [(100, 70, 16, 32, False), (37, 300, 8, 64, True),
                                               (512, 2048, 512, 2048, False)])
def test_csr_to_tiled_oracle_matches_csr2tiledcsr(M, K, TR, TC, shuffle):
    # csr2tiledcsr (source/src/main.cu:499-588) restated with numpy: tiles in
    # row-major order, rows in order, each row's entries in CSR order
    rng = np.random.default_rng(M + K)
    rp, col, val = _random_csr(rng, M, K, 0.05, shuffle)
    acc, toff, tcol, tval = O.csr_to_tiled(rp, col, val, M, K, TR, TC)
    Kt = (K + TC - 1) // TC
    T = ((M + TR - 1) // TR) * Kt
    buckets = [[] for _ in range(T)]
    for i in range(M):
        for j in range(rp[i], rp[i + 1]):
            buckets[(i // TR) * Kt + col[j] // TC].append((i % TR, col[j] % TC, val[j]))
    assert np.array_equal(acc, np.concatenate([[0], np.cumsum([len(b) for b in buckets])]))
    flat = [e for b in buckets for e in b]
    assert np.array_equal(tcol, np.array([e[1] for e in flat], np.int32).reshape(-1))
    assert np.array_equal(tval, np.array([e[2] for e in flat], np.float32).reshape(-1))
    for t, b in enumerate(buckets):
        rows = np.array([e[0] for e in b], np.int64)
        exp = [int((rows < j).sum()) for j in range(TR + 1)]
        assert np.array_equal(toff[t], exp)


def test_symbolic_mask_from_cluster_counts():
    """The identity behind the planned symbolic pass, in numpy: for a row
    with consensus c, added columns (row and not c) and removed columns (c
    and not row), the per-column count of the row's B masks is
    count(c) + count(added) - count(removed); it never drops below zero on
    the way (removed columns are all in c), and its nonzeros are the OR mask
    of the walk."""
    import numpy as np
    from bitwise_spgemm_gb300 import workloads as W
    rng = np.random.default_rng(3)
    A, _, near = W.clustered_bits(200, 300, n_proto=4, p_proto=0.1, p_flip=0.02, seed_proto=3, seed_rows=4)
    Bm = (rng.random((300, 90)) < 0.05).astype(np.int64)
    cons = np.stack([A[near == c].mean(axis=0) > 0.5 for c in range(4)])  # majority per cluster
    Ai = A.astype(np.int64)
    for i in range(A.shape[0]):
        c = cons[near[i]]
        add = (A[i] & ~c).astype(np.int64)
        rem = (c & ~A[i]).astype(np.int64)
        n_c = c.astype(np.int64) @ Bm
        assert np.all(n_c - rem @ Bm >= 0)
        n = n_c + add @ Bm - rem @ Bm
        assert np.array_equal(n, Ai[i] @ Bm)
        assert np.array_equal(n > 0, (Ai[i][:, None] * Bm).max(axis=0) > 0)
