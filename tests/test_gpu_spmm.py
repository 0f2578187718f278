"""SpMM on the GPU against the oracle (FP32 order-exact and FP64) and the
reference fixtures.

Tolerances: integer-valued B must match bit for bit.  Otherwise the error
of every element is measured against the FP64 oracle relative to the scale
of its summation bound, |C - C64| / (|A||B|)_ij, and must be ≤ 1e-5 for FP32
B (the relative tolerance of the reference's check(),
backup/bit_wise_gemm.cu:24); BF16/FP16 B is exact in FP32 so the same bound
holds against the FP64 product of the rounded B.
"""
import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import bf16_dev, words_dev

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _check_f64(C, words, K, Bf32, tol=TOL):
    C64 = O.spmm_f64(words, K, Bf32)
    Cabs = O.spmm_abs_f64(words, K, Bf32)
    mx, mean, mxn = O.rel_errors(C, C64, Cabs)
    assert mx <= tol, (mx, mean, mxn)
    return mx, mean, mxn


def test_reference_fixture_bit_exact(golden):
    A = golden["spmm_A01"].astype(bool)
    words = W.pack_bits(A)
    wd = words_dev(words)
    for bkey, ckey in (("spmm_B_int", "spmm_C_int_ref"), ("spmm_B_normal", "spmm_C_normal_ref")):
        C = ops.spmm(wd, A.shape[1], torch.from_numpy(golden[bkey]).cuda()).cpu().numpy()
        # ascending-column FP32 sums: the reference's own order, bit for bit
        assert np.array_equal(C, golden[ckey]), bkey


def test_config1_bit_exact():
    cfg = W.config1()
    wd = words_dev(cfg["words"])
    B = torch.from_numpy(cfg["B"]).cuda()
    C = ops.spmm(wd, cfg["K"], B).cpu().numpy()
    ref = O.spmm_f32(cfg["words"], cfg["K"], cfg["B"])
    assert np.array_equal(C, ref)
    assert np.array_equal(C.astype(np.float64), O.spmm_f64(cfg["words"], cfg["K"], cfg["B"]))
    # the plan path gives the same integers
    plan = ops.Plan(wd, cfg["K"], mode=capi.PLAN_PROTO)
    C2 = ops.spmm(wd, cfg["K"], B, plan=plan).cpu().numpy()
    assert np.array_equal(C2, ref)


@pytest.fixture(scope="module")
def cfg2():
    return W.config2()


def test_config2_plan_and_tolerance(cfg2):
    words, K, Bn = cfg2["words"], cfg2["K"], cfg2["B"]
    wd = words_dev(words)
    B = torch.from_numpy(Bn).cuda()
    plan = ops.Plan(wd, K)
    info = plan.info()
    assert info["mode"] == capi.PLAN_PROTO
    assert info["n_proto"] >= 64 and info["n_proto"] <= 80
    # the delta lists are a small fraction of the set bits
    assert info["delta_nnz"] + info["proto_nnz"] < 0.1 * info["nnz"]
    C = ops.spmm(wd, K, B, plan=plan)
    Cd = ops.spmm(wd, K, B)
    _check_f64(C.cpu().numpy(), words, K, Bn)
    _check_f64(Cd.cpu().numpy(), words, K, Bn)
    # deterministic
    assert torch.equal(C, ops.spmm(wd, K, B, plan=plan))
    # integer B through the plan: bit-exact even with subtractions
    Bi = np.random.default_rng(12).integers(-8, 9, (K, 512)).astype(np.float32)
    Ci = ops.spmm(wd, K, torch.from_numpy(Bi).cuda(), plan=plan).cpu().numpy()
    assert np.array_equal(Ci.astype(np.float64), O.spmm_f64(words, K, Bi))


@pytest.mark.parametrize("M,K,N,p", [(1, 1, 1, 1.0), (37, 45, 7, 0.3), (64, 1000, 130, 0.1),
                                     (300, 97, 512, 0.05), (128, 64, 1024, 0.5),
                                     (17, 4096, 2048, 0.02)])
@pytest.mark.parametrize("bdt", ["f32", "bf16", "f16"])
def test_random_shapes(M, K, N, p, bdt):
    rng = np.random.default_rng(M * 31 + K + N)
    bits = rng.random((M, K)) < p
    bits[0] = False  # empty row
    words = W.pack_bits(bits)
    Bf = rng.standard_normal((K, N)).astype(np.float32)
    if bdt == "f32":
        B = torch.from_numpy(Bf).cuda()
    elif bdt == "bf16":
        b16 = W.f32_to_bf16_bits(Bf)
        Bf = W.bf16_bits_to_f32(b16)
        B = bf16_dev(b16)
    else:
        B = torch.from_numpy(Bf).half().cuda()
        Bf = B.float().cpu().numpy()
    C = ops.spmm(words_dev(words), K, B).cpu().numpy()
    assert np.all(C[0] == 0)
    _check_f64(C, words, K, Bf)
    if bdt == "f32":
        assert np.array_equal(C, O.spmm_f32(words, K, Bf))


def test_strided_operands():
    rng = np.random.default_rng(5)
    M, K, N = 100, 300, 96
    bits = rng.random((M, K)) < 0.1
    words = W.pack_bits(bits)
    Bbig = torch.from_numpy(rng.standard_normal((K, N + 40)).astype(np.float32)).cuda()
    B = Bbig[:, 8:8 + N]  # ldb = N + 40, 32-byte offset
    Cbig = torch.full((M, N + 4), 7.0, device="cuda")
    C = Cbig[:, :N]
    ops.spmm(words_dev(words), K, B, out=C)
    ref = O.spmm_f32(words, K, B.contiguous().cpu().numpy())
    assert np.array_equal(C.cpu().numpy(), ref)
    assert torch.all(Cbig[:, N:] == 7.0)
    # unaligned B pointer (offset 1 element) takes the lane-per-column path
    B1 = Bbig[:, 1:1 + N]
    C1 = ops.spmm(words_dev(words), K, B1).cpu().numpy()
    assert np.array_equal(C1, O.spmm_f32(words, K, B1.contiguous().cpu().numpy()))


def test_heavy_rows_compensated():
    rng = np.random.default_rng(7)
    M, K, N = 8, 20000, 64
    bits = rng.random((M, K)) < 0.6  # ~12000 set bits per row (> 4096)
    words = W.pack_bits(bits)
    Bf = (rng.standard_normal((K, N)) * 1e3 + 1.0).astype(np.float32)
    C = ops.spmm(words_dev(words), K, torch.from_numpy(Bf).cuda()).cpu().numpy()
    mx, _, _ = _check_f64(C, words, K, Bf)
    # compensated sums are much closer to FP64 than the plain FP32 walk
    C32 = O.spmm_f32(words, K, Bf)
    C64 = O.spmm_f64(words, K, Bf)
    assert np.abs(C - C64).max() < 0.5 * np.abs(C32 - C64).max()


def test_dense_prototypes_compensated():
    """Prototypes with more than 4096 set bits: their sums P[c] are formed
    with TwoSum pairs, so clustered rows stay as close to FP64 as the
    compensated direct walk, and integer-valued B stays exact."""
    rng = np.random.default_rng(11)
    M, K, N = 256, 16384, 256
    A, _, _ = W.clustered_bits(M, K, n_proto=4, p_proto=0.4, p_flip=0.002, seed_proto=12, seed_rows=13)
    words = W.pack_bits(A)
    wd = words_dev(words)
    plan = ops.Plan(wd, K, mode=capi.PLAN_PROTO)
    assert plan.info()["mode"] == capi.PLAN_PROTO and plan.info()["n_proto"] >= 1
    Bf = (rng.standard_normal((K, N)) * 1e3 + 1.0).astype(np.float32)
    C = ops.spmm(wd, K, torch.from_numpy(Bf).cuda(), plan=plan).cpu().numpy()
    assert capi.device_status() == 0
    _check_f64(C, words, K, Bf)
    C64 = O.spmm_f64(words, K, Bf)
    C32 = O.spmm_f32(words, K, Bf)
    assert np.abs(C - C64).max() < 0.5 * np.abs(C32 - C64).max()
    Bi = rng.integers(-8, 9, (K, N)).astype(np.float32)
    Ci = ops.spmm(wd, K, torch.from_numpy(Bi).cuda(), plan=plan).cpu().numpy()
    assert np.array_equal(Ci.astype(np.float64), O.spmm_f64(words, K, Bi))


def test_empty_and_degenerate():
    wd = torch.zeros((0, 2), dtype=torch.int32, device="cuda")
    B = torch.randn(40, 8, device="cuda")
    assert ops.spmm(wd, 40, B).shape == (0, 8)
    wd = torch.zeros((5, 0), dtype=torch.int32, device="cuda")
    C = ops.spmm(wd, 0, torch.zeros((0, 8), device="cuda"))
    assert torch.all(C == 0)
    # all-zero A, plan with no clusters
    wd = torch.zeros((64, 4), dtype=torch.int32, device="cuda")
    plan = ops.Plan(wd, 128)
    assert plan.info()["mode"] == capi.PLAN_DIRECT
    C = ops.spmm(wd, 128, torch.randn(128, 16, device="cuda"), plan=plan)
    assert torch.all(C == 0)


def test_plan_errors():
    wd = torch.zeros((64, 4), dtype=torch.int32, device="cuda")
    plan = ops.Plan(wd, 128)
    with pytest.raises(capi.BspError):
        ops.spmm(wd[:32], 128, torch.randn(128, 16, device="cuda"), plan=plan)
    # proto plan with too-small workspace is rejected
    rng = np.random.default_rng(3)
    A, _, _ = W.clustered_bits(512, 1024, n_proto=4, p_proto=0.2)
    words = W.pack_bits(A)
    wdp = words_dev(words)
    plan = ops.Plan(wdp, 1024, mode=capi.PLAN_PROTO)
    assert plan.info()["mode"] == capi.PLAN_PROTO
    need = plan.workspace_bytes(64, preferred=False)  # the minimum: prototype sums
    ws = torch.empty(need - 300, dtype=torch.uint8, device="cuda")
    import ctypes as C
    Bt = torch.randn(1024, 64, device="cuda")
    Ct = torch.empty(512, 64, device="cuda")
    st = capi.lib().bsp_spmm(C.c_void_p(wdp.data_ptr()), 512, 1024, C.c_void_p(Bt.data_ptr()), 0, 64,
                             64, C.c_void_p(Ct.data_ptr()), 64, plan.handle, C.c_void_p(ws.data_ptr()),
                             ws.numel(), None)
    assert st == -3
    _ = rng


def test_clustered_small_plans_all_modes():
    A, _, _ = W.clustered_bits(2048, 2048, n_proto=16, p_proto=0.1, p_flip=0.01, seed_proto=21,
                               seed_rows=22)
    words = W.pack_bits(A)
    wd = words_dev(words)
    Bf = np.random.default_rng(23).standard_normal((2048, 256)).astype(np.float32)
    B = torch.from_numpy(Bf).cuda()
    outs = []
    for mode in (capi.PLAN_AUTO, capi.PLAN_DIRECT, capi.PLAN_PROTO):
        plan = ops.Plan(wd, 2048, mode=mode)
        C = ops.spmm(wd, 2048, B, plan=plan).cpu().numpy()
        _check_f64(C, words, 2048, Bf)
        outs.append(C)
    b16 = W.f32_to_bf16_bits(Bf)
    plan = ops.Plan(wd, 2048, mode=capi.PLAN_PROTO)
    C = ops.spmm(wd, 2048, bf16_dev(b16), plan=plan).cpu().numpy()
    _check_f64(C, words, 2048, W.bf16_bits_to_f32(b16))


@pytest.mark.parametrize("N", [8, 520, 1536, 2056])
@pytest.mark.parametrize("bdt", ["f32", "bf16", "f16"])
def test_proto_bulk_mixed_rows(N, bdt):
    """Clustered rows (TMA-staged prototype path) mixed with random rows (walked
    directly), several column chunks including a ragged last one."""
    rng = np.random.default_rng(N)
    A, _, _ = W.clustered_bits(1200, 3000, n_proto=6, p_proto=0.08, p_flip=0.004, seed_proto=N,
                               seed_rows=N + 1)
    A[::17] = rng.random((A[::17].shape[0], 3000)) < 0.05  # rows that fit no cluster
    words = W.pack_bits(A)
    wd = words_dev(words)
    Bf = rng.standard_normal((3000, N)).astype(np.float32)
    if bdt == "bf16":
        b16 = W.f32_to_bf16_bits(Bf)
        Bf = W.bf16_bits_to_f32(b16)
        B = bf16_dev(b16)
    elif bdt == "f16":
        B = torch.from_numpy(Bf).half().cuda()
        Bf = B.float().cpu().numpy()
    else:
        B = torch.from_numpy(Bf).cuda()
    plan = ops.Plan(wd, 3000, mode=capi.PLAN_PROTO)
    info = plan.info()
    assert info["mode"] == capi.PLAN_PROTO and info["direct_rows"] > 0
    C = ops.spmm(wd, 3000, B, plan=plan).cpu().numpy()
    assert capi.device_status() == 0
    _check_f64(C, words, 3000, Bf)
    # integer-valued B: the bulk path is exact
    Bi = rng.integers(-8, 9, (3000, N)).astype(np.float32)
    Ci = ops.spmm(wd, 3000, torch.from_numpy(Bi).cuda(), plan=plan).cpu().numpy()
    assert np.array_equal(Ci.astype(np.float64), O.spmm_f64(words, 3000, Bi))
    assert capi.device_status() == 0


@pytest.mark.parametrize("N,bdt", [(512, "f32"), (256, "f32"), (512, "bf16")])
def test_proto_delta_lists_across_the_row_slot(N, bdt):
    """Rows that differ from their prototype in exactly f columns, f from 0 to
    100: the row kernel reads the first 31 delta entries from the row's slot
    and the rest from the list, so counts 30..33 and 62..64 cross both edges.
    Integer-valued B is exact; Gaussian B within the FP32 bound."""
    rng = np.random.default_rng(N + 7)
    K, flips = 4096, [0, 1, 2, 30, 31, 32, 33, 62, 63, 64, 100]
    protos = rng.random((4, K)) < 0.1
    rows = []
    for p in protos:
        for f in flips:
            for _ in range(6):
                r = p.copy()
                idx = rng.choice(K, f, replace=False)
                r[idx] = ~r[idx]
                rows.append(r)
    A = np.array(rows)
    words = W.pack_bits(A)
    wd = words_dev(words)
    plan = ops.Plan(wd, K, mode=capi.PLAN_PROTO)
    info = plan.info()
    assert info["mode"] == capi.PLAN_PROTO and info["delta_nnz"] > 0
    Bi = rng.integers(-8, 9, (K, N)).astype(np.float32)
    if bdt == "bf16":
        Bd = bf16_dev(W.f32_to_bf16_bits(Bi))
    else:
        Bd = torch.from_numpy(Bi).cuda()
    Ci = ops.spmm(wd, K, Bd, plan=plan).cpu().numpy()
    assert capi.device_status() == 0
    assert np.array_equal(Ci.astype(np.float64), O.spmm_f64(words, K, Bi))
    Bf = rng.standard_normal((K, N)).astype(np.float32)
    if bdt == "bf16":
        b16 = W.f32_to_bf16_bits(Bf)
        Bf, Bd = W.bf16_bits_to_f32(b16), bf16_dev(b16)
    else:
        Bd = torch.from_numpy(Bf).cuda()
    C = ops.spmm(wd, K, Bd, plan=plan).cpu().numpy()
    _check_f64(C, words, K, Bf)


def test_plan_destroy_async_in_a_loop():
    """Plans built, used and released in stream order, back to back on one
    stream without a host wait between steps (the serving-loop pattern):
    every step's C is exact on integer B."""
    rng = np.random.default_rng(31)
    A, _, _ = W.clustered_bits(1024, 2048, n_proto=8, p_proto=0.08, p_flip=0.004, seed_proto=31,
                               seed_rows=32)
    words = W.pack_bits(A)
    wd = words_dev(words)
    outs = []
    Bs = [rng.integers(-8, 9, (2048, 256)).astype(np.float32) for _ in range(4)]
    for Bi in Bs:
        plan = ops.Plan(wd, 2048, mode=capi.PLAN_PROTO)
        outs.append(ops.spmm(wd, 2048, torch.from_numpy(Bi).cuda(), plan=plan))
        plan.close_async()
    torch.cuda.synchronize()
    for Bi, C in zip(Bs, outs):
        assert np.array_equal(C.cpu().numpy().astype(np.float64), O.spmm_f64(words, 2048, Bi))
    assert capi.device_status() == 0


_PATHS_SCRIPT = r"""
import json, sys, hashlib
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import words_dev
rng = np.random.default_rng(41)
A, _, _ = W.clustered_bits(2048, 3000, n_proto=12, p_proto=0.08, p_flip=0.003, seed_proto=41, seed_rows=42)
A[::7] = rng.random((A[::7].shape[0], 3000)) < 0.004   # sparser than 1/64: direct hashing
A[3::11] = rng.random((A[3::11].shape[0], 3000)) < 0.5  # dense rows
wd = words_dev(W.pack_bits(A))
plan = ops.Plan(wd, 3000)
Bi = torch.from_numpy(rng.integers(-8, 9, (3000, 64)).astype(np.float32)).cuda()
C = ops.spmm(wd, 3000, Bi, plan=plan).cpu().numpy()
print(json.dumps({"info": plan.info(), "C": hashlib.sha1(C.tobytes()).hexdigest()}))
"""


def test_minhash_paths_agree():
    """The signature kernel's column-order scan and its direct hashing of
    every set bit give the same MinHash values, hence the same plan (same
    prototypes and delta lists) and the same C, bit for bit."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for direct in ("0", "1"):
        env = dict(os.environ, BSP_MINHASH_DIRECT=direct)
        r = subprocess.run([sys.executable, "-c", _PATHS_SCRIPT, root], env=env, capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(json.loads(r.stdout.strip().splitlines()[-1]))
    assert outs[0] == outs[1]
    assert outs[0]["info"]["mode"] == capi.PLAN_PROTO


def test_plan_with_many_rows():
    """More than 32768 rows: the plan numbers its clusters and sizes its row
    lists with the multi-CTA scans.  Integer B through the plan is exact, and
    the planned symbolic mask equals the walk."""
    rng = np.random.default_rng(77)
    M, K, N = 40000, 512, 64
    A, _, _ = W.clustered_bits(M, K, n_proto=20, p_proto=0.1, p_flip=0.004, seed_proto=77, seed_rows=78)
    A[::101] = rng.random((A[::101].shape[0], K)) < 0.05
    words = W.pack_bits(A)
    wd = words_dev(words)
    plan = ops.Plan(wd, K, mode=capi.PLAN_PROTO)
    info = plan.info()
    assert info["mode"] == capi.PLAN_PROTO and info["n_proto"] >= 20 and info["delta_nnz"] > 0
    Bi = rng.integers(-8, 9, (K, N)).astype(np.float32)
    C = ops.spmm(wd, K, torch.from_numpy(Bi).cuda(), plan=plan).cpu().numpy()
    assert np.array_equal(C.astype(np.float64), O.spmm_f64(words, K, Bi))
    Bm = W.pack_bits(rng.random((K, 96)) < 0.05)
    bd = words_dev(Bm)
    s1 = ops.symbolic_rows(wd, K, bd, 96, plan=plan)
    s0 = ops.symbolic_rows(wd, K, bd, 96)
    assert torch.equal(s1, s0)
    assert capi.device_status() == 0


def test_probe_gather_runs_and_checks_its_arguments():
    """The L2 gather roof probe (bsp_probe_gather): a small launch with every
    slice size returns OK and leaves the sink untouched (the gathered sum is
    never the impossible value); indices past the buffer are skipped."""
    import ctypes
    rows, row_bytes = 256, 2048
    buf = torch.randn(rows * row_bytes // 4, device="cuda")
    n_warps, per_warp = 64, 40
    idx = torch.randint(0, rows + 8, (n_warps * per_warp,), device="cuda", dtype=torch.int32)
    sink = torch.zeros(n_warps, device="cuda")
    for sb in (512, 1024, 2048):
        st = capi.lib().bsp_probe_gather(ctypes.c_void_p(buf.data_ptr()), rows, row_bytes,
                                         ctypes.c_void_p(idx.data_ptr()), n_warps, per_warp, sb,
                                         ctypes.c_void_p(sink.data_ptr()), None)
        assert st == 0
    torch.cuda.synchronize()
    assert float(sink.abs().max()) == 0.0
    assert capi.lib().bsp_probe_gather(ctypes.c_void_p(buf.data_ptr()), rows, 1024,
                                       ctypes.c_void_p(idx.data_ptr()), n_warps, per_warp, 2048,
                                       ctypes.c_void_p(sink.data_ptr()), None) == -2


_SUMS_SCRIPT = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
A, _, _ = W.clustered_bits(1024, 3000, n_proto=5, p_proto=0.08, p_flip=0.004, seed_proto=5, seed_rows=6)
words = W.pack_bits(A)
wd = torch.from_numpy(np.ascontiguousarray(words).view(np.int32)).cuda()
plan = ops.Plan(wd, 3000, mode=capi.PLAN_PROTO)
B = np.random.default_rng(7).integers(-8, 9, (3000, 520)).astype(np.float32)
C = ops.spmm(wd, 3000, torch.from_numpy(B).cuda(), plan=plan)
torch.cuda.synchronize()
assert capi.device_status() == 0
np.save(sys.argv[2], C.cpu().numpy())
"""


@pytest.mark.parametrize("form", ["-1", "0", "1"])
def test_prototype_sum_forms(tmp_path, form):
    """Each prototype-sum form (BSP_SUMS_BULK: -1 the cluster form over the
    column lists, n >= 0 a bulk-copy staging shape; read once per process, so
    each runs in a child process) gives the exact integer product."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = tmp_path / "C.npy"
    env = dict(os.environ, BSP_SUMS_BULK=form)
    r = subprocess.run([sys.executable, "-c", _SUMS_SCRIPT, root, str(out)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    A, _, _ = W.clustered_bits(1024, 3000, n_proto=5, p_proto=0.08, p_flip=0.004, seed_proto=5, seed_rows=6)
    B = np.random.default_rng(7).integers(-8, 9, (3000, 520)).astype(np.float32)
    assert np.array_equal(np.load(out).astype(np.float64), O.spmm_f64(W.pack_bits(A), 3000, B))


_SLOT_SCRIPT = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
A, _, _ = W.clustered_bits(2048, 4096, n_proto=12, p_proto=0.05, p_flip=0.004, seed_proto=8, seed_rows=9)
wd = torch.from_numpy(np.ascontiguousarray(W.pack_bits(A)).view(np.int32)).cuda()
B = torch.from_numpy(np.random.default_rng(10).standard_normal((4096, 512), dtype=np.float32)).cuda()
outs = []
for _ in range(2):  # two plans of the same A: rows of equal delta count may take other slots
    plan = ops.Plan(wd, 4096, mode=capi.PLAN_PROTO)
    outs.append(ops.spmm(wd, 4096, B, plan=plan))
torch.cuda.synchronize()
assert capi.device_status() == 0
assert torch.equal(outs[0], outs[1])
np.save(sys.argv[2], outs[0].cpu().numpy())
"""


def test_row_slot_order_does_not_change_results(tmp_path):
    """The row kernel's slot order (longest delta lists first, equal lengths
    in any order) and the index-order walk through the list bounds
    (BSP_SLOT_LISTS=0) give the same FP32 C bit for bit, and so do two plans
    of the same A."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for flag in ("1", "0"):
        out = tmp_path / ("C%s.npy" % flag)
        env = dict(os.environ, BSP_SLOT_LISTS=flag)
        r = subprocess.run([sys.executable, "-c", _SLOT_SCRIPT, root, str(out)], env=env, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(np.load(out))
    assert np.array_equal(outs[0], outs[1])
