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

    np.savez_compressed(OUT, **fx)
    print("wrote", OUT, {k: getattr(v, "shape", ()) for k, v in fx.items()})


if __name__ == "__main__":
    main()
