"""Generate the golden fixtures in this folder from the reference's own code.

Runs the reference kernels and CPU check built by oracle/build_ref.py (the
reference checkout must be present — this container only) on small seeded
inputs and stores inputs + reference outputs in ``reference_small.npz``.
Tests on machines without the reference compare the oracle and the CUDA
library against these frozen outputs.

Usage: python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref as R  # noqa: E402
from bitwise_spgemm_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_small.npz")


def main():
    if not R.build_ref.available():
        raise SystemExit("reference checkout not found; fixtures need the reference's own code")
    rng = np.random.default_rng(20240601)
    fx = {}
    # 1. dense2bitmask (source/src/main.cu:591-628): values incl. -0.0, NaN, inf, denormals
    M, K, TR = 128, 96, 64
    dense = np.where(rng.random((M, K)) < 0.15, rng.standard_normal((M, K)), 0).astype(np.float32)
    special = np.array([-0.0, np.nan, np.inf, -np.inf, 1e-42, -1e-42], np.float32)
    pos = rng.choice(M * K, size=48, replace=False)
    dense.reshape(-1)[pos] = np.resize(special, 48)
    fx["pack_dense"] = dense
    fx["pack_tile_rows"] = np.int32(TR)
    fx["pack_words_msb"] = R.dense2bitmask(dense, TR)

    # 2. generate_groups_large (main.cu:50-247) on int8-valued data, 256 rows x 128 cols, tiles of 64 rows
    M, K, TR = 256, 128, 64
    bits = rng.random((M, K)) < 0.1
    gdense = np.where(bits, rng.integers(1, 100, (M, K)), 0).astype(np.float32)
    gw = R.dense2bitmask(gdense, TR)
    g = R.generate_groups_large(gw, gdense, TR)
    fx["group_dense"] = gdense
    fx["group_tile_rows"] = np.int32(TR)
    fx["group_words_msb"] = gw
    fx["group_id_ref"] = g["group_id"]          # spilled rows carry 2 (= MAX_GROUP_NUM), main.cu:184
    fx["group_mask_ref"] = g["group_mask"]
    fx["group_val_ref"] = g["group_val"]
    fx["group_nnz_ref"] = g["nnz"]

    # 3. group2dense (main.cu:829-850): tile-major inputs built from the grouping above
    T = (M // TR) * (K // 32)
    gvals = rng.standard_normal((T, 2, 32)).astype(np.float32)
    Kw = K // 32
    gid_tm = np.zeros(T * TR, np.int32)
    bm_tm = np.zeros(T * TR, np.uint32)
    for t in range(T):
        rb, w = divmod(t, Kw)
        gid_tm[t * TR:(t + 1) * TR] = np.where(g["group_id"][rb * TR:(rb + 1) * TR, w] == 2, -1,
                                               g["group_id"][rb * TR:(rb + 1) * TR, w])
        bm_tm[t * TR:(t + 1) * TR] = gw[rb * TR:(rb + 1) * TR, w]
    fx["g2d_values"] = gvals
    fx["g2d_dense_ref"] = R.group2dense(gvals, gid_tm, bm_tm, M, K, TR)

    # 4. uint8_layout_trans (backup/layout_trans.cu:87-97)
    v = rng.integers(0, 256, (16, 64)).astype(np.uint8)
    fx["planes_u8"] = v
    fx["planes_ref"] = R.uint8_layout_trans(v)

    # 5. uint8_spmm_2d_1d (layout_trans.cu:158-171) on 0/1 masks: integer and N(0,1) B
    A01 = (rng.random((32, 1024)) < 0.1).astype(np.uint8)
    planes = R.uint8_layout_trans(A01)
    Bi = rng.integers(-8, 9, (1024, 64)).astype(np.float32)
    Bn = rng.standard_normal((1024, 64)).astype(np.float32)
    fx["spmm_A01"] = A01
    fx["spmm_B_int"] = Bi
    fx["spmm_B_normal"] = Bn
    fx["spmm_C_int_ref"] = R.uint8_spmm(planes, Bi)
    fx["spmm_C_normal_ref"] = R.uint8_spmm(planes, Bn)

    # 6. multi-bit uint8 values through all 8 planes (the bit-serial product)
    A8 = np.where(rng.random((8, 256)) < 0.2, rng.integers(0, 256, (8, 256)), 0).astype(np.uint8)
    Bs = rng.integers(-4, 5, (256, 32)).astype(np.float32)
    fx["bitserial_A_u8"] = A8
    fx["bitserial_B"] = Bs
    fx["bitserial_C_ref"] = R.uint8_spmm(R.uint8_layout_trans(A8), Bs)

    # 7. check() (backup/bit_wise_gemm.cu:13-32) verdicts on the C above (True) and a perturbed C (False)
    Cgood = fx["spmm_C_normal_ref"]
    Cbad = Cgood.copy()
    Cbad[3, 5] += 1e-2 * max(1.0, abs(float(Cbad[3, 5])))
    fx["check_good"] = np.bool_(R.check(A01.astype(np.float32), Bn, Cgood))
    fx["check_bad"] = np.bool_(R.check(A01.astype(np.float32), Bn, Cbad))
    fx["check_C_bad"] = Cbad

    # The sections below draw from their own generator, so the keys above keep their values.
    rng = np.random.default_rng(20261204)

    # 8. csr2tiledcsr (main.cu:499-588), three tile shapes; empty rows, an empty
    #    tile and entries within a row in CSR (column) order
    for name, (M, K, th, tw, p) in {"256x256": (768, 512, 256, 256, 0.03),
                                    "64x64": (192, 128, 64, 64, 0.08),
                                    "32x128": (96, 384, 32, 128, 0.05)}.items():
        A = rng.random((M, K)) < p
        A[5] = False
        A[:th, :tw] = False  # tile 0 empty
        rp = np.concatenate([[0], np.cumsum(A.sum(1))]).astype(np.int32)
        col = np.nonzero(A)[1].astype(np.int32)
        val = rng.standard_normal(len(col)).astype(np.float32)
        t = R.csr2tiledcsr(rp, col, val, M, K, th, tw)
        fx["c2t_%s_row_ptr" % name] = rp
        fx["c2t_%s_col" % name] = col
        fx["c2t_%s_val" % name] = val
        fx["c2t_%s_shape" % name] = np.array([M, K, th, tw], np.int32)
        for k in ("tile_nnz_acc", "tiled_offset", "tiled_col", "tiled_val", "tile_row_nnz"):
            fx["c2t_%s_%s" % (name, k)] = t[k]

    # 9. pre_spgemm (transform.cuh:984-1157): the symbolic output mask of A·B
    #    with B a bitmap, and first-fit grouping of the output rows (2 groups).
    #    TILE_HEIGHT = SPLIT_K = K (the kernel's only race-free shape, see
    #    oracle/ref_emu_out.cpp); dense enough that rows spill.
    for name, (M, N, t, pa, pb) in {"256": (512, 128, 256, 0.02, 0.05),
                                    "64": (256, 96, 64, 0.05, 0.1)}.items():
        K = t
        A = rng.random((M, K)) < pa
        A[7] = False
        Bd = (rng.random((K, N)) < pb).astype(np.float32)
        bw = R.dense2bitmask(Bd, 64)  # B's masks as main() builds them (MSB-first)
        rp = np.concatenate([[0], np.cumsum(A.sum(1))]).astype(np.int32)
        col = np.nonzero(A)[1].astype(np.int32)
        tl = R.csr2tiledcsr(rp, col, np.ones(len(col), np.float32), M, K, t, t)
        o = R.pre_spgemm(bw, tl, M, K, N, t)
        fx["pre_%s_A_words" % name] = W.pack_bits(A)
        fx["pre_%s_B_words_msb" % name] = bw
        fx["pre_%s_shape" % name] = np.array([M, K, N, t], np.int32)
        fx["pre_%s_c_bits" % name] = o["c_bits"]
        fx["pre_%s_group_idx" % name] = o["group_idx"]
        fx["pre_%s_group_mask" % name] = o["group_mask"]
        fx["pre_%s_nnz" % name] = o["nnz"]

    # 10. coo2bmp_noTuple_d (main.cu:692-779, mm.h:83-144): 8x8 bitmap tiles,
    #     tile coordinates and popcount offsets, from COO entries in any order;
    #     ragged edges (M, K not multiples of 8) and an all-zero band
    for name, (M, K, p) in {"64x64": (64, 64, 0.1), "37x91": (37, 91, 0.2),
                            "200x130": (200, 130, 0.03)}.items():
        A = rng.random((M, K)) < p
        A[8:16] = False
        r, c = np.nonzero(A)
        perm = rng.permutation(len(r))
        bmp, tr, tc, ix, _ = R.coo2bmp(r[perm], c[perm], np.ones(len(r), np.float32), M, K)
        fx["bmp_%s_words" % name] = W.pack_bits(A)
        fx["bmp_%s_shape" % name] = np.array([M, K], np.int32)
        fx["bmp_%s_bmp" % name] = bmp
        fx["bmp_%s_tile_row" % name] = tr
        fx["bmp_%s_tile_col" % name] = tc
        fx["bmp_%s_idx" % name] = ix

    # 11. the 1024x1024 Bernoulli(0.1) matrix of the small plain SpMM (seed 0):
    #     the reference's packing (MSB-first) and row groups at its own
    #     TILE_HEIGHT of 512 rows and MAX_GROUP_NUM of 2
    c1 = W.config1()
    A1 = W.unpack_bits(c1["words"], c1["K"]).astype(np.float32)
    w1 = R.dense2bitmask(A1, 512)
    g1 = R.generate_groups_large(w1, A1, 512)
    fx["c1_words_msb"] = w1
    fx["c1_group_id_ref"] = g1["group_id"]
    fx["c1_group_mask_ref"] = g1["group_mask"]
    fx["c1_group_nnz_ref"] = g1["nnz"]

    np.savez_compressed(OUT, **fx)
    print("wrote", OUT, {k: getattr(v, "shape", ()) for k, v in fx.items()})


if __name__ == "__main__":
    main()
