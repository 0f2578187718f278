"""Batched tensor-core SpMM (persistent for N ≤ 128) against the oracle: problems of uneven
M, K and density, column blocking, empty problems and CUDA-graph replay.
Scaled error against FP64 ≤ 1e-4 (BF16 products are exact, FP32
accumulation), integer-valued B exact."""
import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from gpu_util import bf16_dev

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _problems(n, N, seed, integer=False, kmax=1024):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        M = int(32 * rng.integers(1, 40))
        K = int(32 * rng.integers(1, kmax // 32))
        d = float(rng.uniform(0.01, 0.3))
        words = W.pack_bits(rng.random((M, K)) < d)
        Bf = (rng.integers(-8, 9, (K, N)) if integer else rng.standard_normal((K, N))).astype(np.float32)
        b16 = W.f32_to_bf16_bits(Bf)
        out.append((words, K, b16))
    return out


def _run(probs, N):
    dev = []
    for words, K, b16 in probs:
        wd = torch.from_numpy(np.ascontiguousarray(words).view(np.int32)).cuda()
        dev.append((wd, K, bf16_dev(b16), torch.full((words.shape[0], N), float("nan"), device="cuda")))
    return dev


@pytest.mark.parametrize("N", [40, 64, 128, 200, 520])
def test_batched_matches_oracle(N):
    probs = _problems(24, N, seed=N)
    dev = _run(probs, N)
    batch = ops.Batch(dev)
    batch.run()
    torch.cuda.synchronize()
    assert capi.device_status() == 0
    for (words, K, b16), (_, _, _, Cd) in zip(probs, dev):
        Bx = W.bf16_bits_to_f32(b16)
        C = Cd.cpu().numpy()
        mx, _, _ = O.rel_errors(C, O.spmm_f64(words, K, Bx), O.spmm_abs_f64(words, K, Bx))
        assert mx <= TOL


def test_batched_integer_exact_and_graph_replay():
    N = 128
    probs = _problems(16, N, seed=5, integer=True)
    dev = _run(probs, N)
    batch = ops.Batch(dev)
    batch.run()  # first run outside capture
    torch.cuda.synchronize()
    for _, _, _, Cd in dev:
        Cd.fill_(float("nan"))
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            batch.run()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert capi.device_status() == 0
    for (words, K, b16), (_, _, _, Cd) in zip(probs, dev):
        assert np.array_equal(Cd.cpu().numpy().astype(np.float64), O.spmm_f64(words, K, W.bf16_bits_to_f32(b16)))


def test_batched_empty_reduction_and_validation():
    N = 128
    wd = torch.zeros((64, 0), dtype=torch.int32, device="cuda")
    Bz = torch.zeros((0, N), dtype=torch.bfloat16, device="cuda")
    Cz = torch.full((64, N), 3.0, device="cuda")
    probs = _problems(3, N, seed=9)
    dev = _run(probs, N) + [(wd, 0, Bz, Cz)]
    batch = ops.Batch(dev)
    batch.run()
    torch.cuda.synchronize()
    assert torch.all(Cz == 0)
    # FP32 B is not a batch type; N not a multiple of 8 is refused
    with pytest.raises(capi.BspError):
        ops.Batch([(dev[0][0], dev[0][1], dev[0][2].float(), dev[0][3])])
    Bodd = torch.zeros((dev[0][1], 12), dtype=torch.bfloat16, device="cuda")
    with pytest.raises(capi.BspError):
        ops.Batch([(dev[0][0], dev[0][1], Bodd, torch.zeros((dev[0][0].shape[0], 12), device="cuda"))])


_PATHS = r"""
import sys, hashlib
import numpy as np, torch
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
import test_gpu_batched as T
from bitwise_spgemm_gb300 import capi, ops
for N in (128, 72, 8):
    probs = T._problems(40, N, seed=100 + N)
    dev = T._run(probs, N)
    batch = ops.Batch(dev)
    batch.run()
    batch.run()  # a second run: the work queue restarts
    torch.cuda.synchronize()
    assert capi.device_status() == 0
    print(N, hashlib.sha1(b"".join(c.cpu().numpy().tobytes() for _, _, _, c in dev)).hexdigest())
"""


def test_persistent_matches_item_per_cta():
    """N ≤ 128 runs on the persistent kernel (work queue, two TMEM
    accumulator sets); the CTA-per-item launch computes the same MMAs in the
    same order, so both give the same C bit for bit (ragged M, N = 72 and 8,
    some problems with one 128-row half)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for persist in ("1", "0"):
        env = dict(os.environ, BSP_BATCH_PERSIST=persist)
        r = subprocess.run([sys.executable, "-c", _PATHS, root], env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(r.stdout.strip().splitlines()[-3:])
    assert outs[0] == outs[1]


def _grad_problems(n, N, seed, integer):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        M = int(32 * rng.integers(1, 48)) + (int(rng.integers(1, 31)) if i % 5 == 3 else 0)  # some ragged M
        K = int(8 * rng.integers(4, 160))
        d = float(rng.uniform(0.01, 0.3))
        A = rng.random((M, K)) < d
        if i == 2:
            A[:, :] = False  # a problem without set bits: dX and dA are zero
        draw = (lambda s: rng.integers(-4, 5, s)) if integer else (lambda s: rng.standard_normal(s))
        X16 = W.f32_to_bf16_bits(draw((K, N)).astype(np.float32))
        G16 = W.f32_to_bf16_bits(draw((M, N)).astype(np.float32))
        out.append((A, W.pack_bits(A), K, X16, G16))
    return out


@pytest.mark.parametrize("N,integer", [(24, True), (64, False), (128, True), (128, False), (264, False)])
def test_batched_grad_matches_oracle(N, integer):
    """dX = Aᵀ·G and dA = (G·Xᵀ) ⊙ A for a batch of uneven problems against
    the FP64 oracle (integer-valued X and G exactly, N(0,1) within the scaled
    tolerance), against the single-problem bsp_spmm_t / bsp_sddmm, and
    stable over two runs."""
    probs = _grad_problems(20, N, seed=N + integer, integer=integer)
    dev = []
    for A, words, K, X16, G16 in probs:
        M = words.shape[0]
        wd = torch.from_numpy(np.ascontiguousarray(words).view(np.int32)).cuda()
        dev.append((wd, K, bf16_dev(X16), bf16_dev(G16), torch.full((K, N), float("nan"), device="cuda"),
                    torch.full((M, K), float("nan"), device="cuda")))
    batch = ops.BatchGrad(dev)
    for run in range(2):
        batch.run()
        torch.cuda.synchronize()
        assert capi.device_status() == 0
        for (A, words, K, X16, G16), (wd, _, Xd, Gd, dXd, dAd) in zip(probs, dev):
            M = words.shape[0]
            X, G = W.bf16_bits_to_f32(X16), W.bf16_bits_to_f32(G16)
            dX, dA = dXd.cpu().numpy(), dAd.cpu().numpy()
            dX64 = O.spmm_t_f64(words, M, K, G)
            vals64 = O.sddmm_f64(words, M, K, G, X)
            assert np.all(dA[~A] == 0.0)
            if integer:
                assert np.array_equal(dX.astype(np.float64), dX64)
                assert np.array_equal(dA[A].astype(np.float64), vals64)
            else:
                mx, _, _ = O.rel_errors(dX, dX64, O.spmm_t_f64(words, M, K, np.abs(G)))
                assert mx <= TOL
                scale = (np.abs(G.astype(np.float64)) @ np.abs(X.astype(np.float64)).T)[A]
                err = np.abs(dA[A] - vals64) / np.where(scale > 0, scale, 1.0)
                assert err.size == 0 or err.max() <= TOL
            if run == 0:
                ref_dX = ops.spmm_t(wd, M, K, Gd).cpu().numpy()
                ref_dA = ops.sddmm(wd, M, K, Gd, Xd).cpu().numpy()
                assert np.abs(dX - ref_dX).max() <= 1e-3 * max(1.0, float(np.abs(ref_dX).max()))
                assert np.abs(dA - ref_dA).max() <= 1e-3 * max(1.0, float(np.abs(ref_dA).max()))
    batch.close()


def test_batched_grad_validation():
    w = torch.zeros((64, 2), dtype=torch.int32, device="cuda")
    X = torch.zeros((60, 128), dtype=torch.bfloat16, device="cuda")
    G = torch.zeros((64, 128), dtype=torch.bfloat16, device="cuda")
    dA = torch.zeros((64, 60), device="cuda")
    with pytest.raises(capi.BspError):  # dA needs K % 8 == 0
        ops.BatchGrad([(w, 60, X, G, None, dA)])
    fwd = ops.Batch([(w, 60, X, torch.zeros((64, 128), device="cuda"))])
    assert capi.lib().bsp_batched_spmm_grad(fwd._h, None) == -1  # BSP_ERR_INVALID_ARG


@pytest.mark.slow
def test_batched_set_real_shapes_against_fp64():
    """Every 32nd problem of the 512-problem batched set itself (M, K
    log-uniform in [64, 4096], density U(0.01, 0.3), N = 128, seeds 7+i):
    forward through the persistent kernel, and the backward pass with the
    set's seeded gradients, against FP64 (BF16 products are exact, FP32
    accumulation: scaled error ≤ 1e-4)."""
    idx = list(range(0, 512, 32))
    probs = [W.config4_problem(i) for i in idx]
    fwd, grad = [], []
    for i, pr in zip(idx, probs):
        M, K = pr["M"], pr["K"]
        wd = torch.from_numpy(np.ascontiguousarray(pr["words"]).view(np.int32)).cuda()
        X = bf16_dev(pr["B"])
        G = bf16_dev(W.config4_grad(pr, i))
        fwd.append((wd, K, X, torch.full((M, 128), float("nan"), device="cuda")))
        grad.append((wd, K, X, G, torch.full((K, 128), float("nan"), device="cuda"),
                     torch.full((M, K), float("nan"), device="cuda")))
    bf, bg = ops.Batch(fwd), ops.BatchGrad(grad)
    bf.run()
    bg.run()
    torch.cuda.synchronize()
    assert capi.device_status() == 0
    for i, pr, f, g in zip(idx, probs, fwd, grad):
        M, K, words = pr["M"], pr["K"], pr["words"]
        X, G = W.bf16_bits_to_f32(pr["B"]), W.bf16_bits_to_f32(W.config4_grad(pr, i))
        mx, _, _ = O.rel_errors(f[3].cpu().numpy(), O.spmm_f64(words, K, X), O.spmm_abs_f64(words, K, X))
        assert mx <= TOL, (i, "Y", mx)
        mx, _, _ = O.rel_errors(g[4].cpu().numpy(), O.spmm_t_f64(words, M, K, G), O.spmm_t_f64(words, M, K, np.abs(G)))
        assert mx <= TOL, (i, "dX", mx)
        A = W.unpack_bits(words, K)
        dA = g[5].cpu().numpy()
        v64 = O.sddmm_f64(words, M, K, G, X)
        sc = (np.abs(G.astype(np.float64)) @ np.abs(X.astype(np.float64)).T)[A]
        assert np.all(dA[~A] == 0.0)
        assert (np.abs(dA[A] - v64) / np.where(sc > 0, sc, 1.0)).max() <= TOL, (i, "dA")


def test_batch_tune_keeps_results_exact():
    """bsp_batch_tune times every shape of the persistent kernel, keeps the
    fastest, and each shape gives the same exact integer products."""
    N = 128
    probs = _problems(20, N, seed=31, integer=True)
    dev = _run(probs, N)
    batch = ops.Batch(dev)
    shape, ms = batch.tune()
    assert 0 <= shape < 4 and ms > 0
    for _, _, _, Cd in dev:
        Cd.fill_(float("nan"))
    batch.run()
    torch.cuda.synchronize()
    assert capi.device_status() == 0
    for (words, K, b16), (_, _, _, Cd) in zip(probs, dev):
        assert np.array_equal(Cd.cpu().numpy().astype(np.float64), O.spmm_f64(words, K, W.bf16_bits_to_f32(b16)))
    # a batch of N > 128 has one form
    probs = _problems(4, 200, seed=32, integer=True)
    dev = _run(probs, 200)
    batch = ops.Batch(dev)
    assert batch.tune()[0] == 0
