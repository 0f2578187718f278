"""Backward pass on the GPU: dX = Aᵀ·G (bsp_spmm_t) and the straight-through
mask gradient dA = (G·Xᵀ) ⊙ A (bsp_sddmm), directly and through the autograd
shim, against the FP64 oracle, a dense PyTorch FP64 gradient and FP64
central finite differences.

Tolerances: integer-valued operands are exact; otherwise every element is
within 1e-4 of FP64 relative to its summation scale (Σ|terms|), inside the
1e-2 bound of the differentiable form."""
import os

import numpy as np
import pytest
import torch

import oracle as O
from bitwise_spgemm_gb300 import capi, ops
from bitwise_spgemm_gb300 import workloads as W
from bitwise_spgemm_gb300.autograd import bitmap_matmul
from gpu_util import bf16_dev, words_dev

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _operand(Af, kind):
    if kind == "bf16":
        b = W.f32_to_bf16_bits(Af)
        return bf16_dev(b), W.bf16_bits_to_f32(b)
    if kind == "f16":
        t = torch.from_numpy(Af).half().cuda()
        return t, t.float().cpu().numpy()
    return torch.from_numpy(Af).cuda(), Af


def _scaled_max(err, scale):
    return float((np.abs(err) / np.where(scale > 0, scale, 1.0)).max()) if err.size else 0.0


@pytest.mark.parametrize("kind", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("tc", ["0", "1"])
@pytest.mark.parametrize("M,K,N,p", [(64, 96, 256, 0.2), (300, 200, 264, 0.1), (513, 1000, 128, 0.05)])
def test_spmm_t(kind, tc, M, K, N, p, monkeypatch):
    if kind == "f32" and tc == "1":
        pytest.skip("FP32 operands stay on CUDA cores")
    monkeypatch.setenv("BSP_TC", tc)
    rng = np.random.default_rng(M * 7 + K + N)
    bits = rng.random((M, K)) < p
    words = W.pack_bits(bits)
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    G, Gx = _operand(rng.standard_normal((M, N)).astype(np.float32), kind)
    dX = ops.spmm_t(wd, M, K, G, plan=plan).cpu().numpy()
    assert capi.device_status() == 0
    ref = O.spmm_t_f64(words, M, K, Gx)
    scale = O.spmm_t_f64(words, M, K, np.abs(Gx))
    assert _scaled_max(dX - ref, scale) <= TOL
    Gi, Gie = _operand(rng.integers(-8, 9, (M, N)).astype(np.float32), kind)
    dXi = ops.spmm_t(wd, M, K, Gi, plan=plan).cpu().numpy()
    assert np.array_equal(dXi.astype(np.float64), O.spmm_t_f64(words, M, K, Gie))


@pytest.mark.parametrize("kind", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("tc", ["0", "1"])
@pytest.mark.parametrize("M,K,N,p", [(64, 96, 256, 0.2), (300, 264, 200, 0.1), (257, 512, 1000, 0.05)])
def test_sddmm(kind, tc, M, K, N, p, monkeypatch):
    if kind == "f32" and tc == "1":
        pytest.skip("FP32 operands stay on CUDA cores")
    monkeypatch.setenv("BSP_TC", tc)
    rng = np.random.default_rng(M + 3 * K + N)
    bits = rng.random((M, K)) < p
    if M > 200:
        bits[:128, :256] = False  # a block without bits: skipped on the tensor cores
    words = W.pack_bits(bits)
    wd = words_dev(words)
    G, Gx = _operand(rng.standard_normal((M, N)).astype(np.float32), kind)
    X, Xx = _operand(rng.standard_normal((K, N)).astype(np.float32), kind)
    dA = ops.sddmm(wd, M, K, G, X).cpu().numpy()
    assert capi.device_status() == 0
    full = Gx.astype(np.float64) @ Xx.astype(np.float64).T
    scale = np.abs(Gx).astype(np.float64) @ np.abs(Xx).astype(np.float64).T
    assert np.all(dA[~bits] == 0)
    assert _scaled_max((dA - full)[bits], scale[bits]) <= TOL
    # the oracle's set-bit order agrees
    vals = O.sddmm_f64(words, M, K, Gx, Xx)
    assert np.allclose(vals, full[bits], rtol=0, atol=1e-9 * max(1.0, np.abs(full).max()))


def _loss64(A, X, G):
    return float(((A @ X) * G).sum())


@pytest.mark.parametrize("kind", ["f32", "bf16"])
@pytest.mark.parametrize("recompute", [False, True])
def test_autograd_against_dense_fp64_and_finite_differences(kind, recompute):
    rng = np.random.default_rng(8)
    M, K, N = 256, 320, 512
    bits = rng.random((M, K)) < 0.1
    Xt, Xx = _operand(rng.standard_normal((K, N)).astype(np.float32), kind)
    Gt, Gx = _operand(rng.standard_normal((M, N)).astype(np.float32), kind)
    mask = torch.from_numpy(bits.astype(np.float32)).cuda().requires_grad_(True)
    X = Xt.clone().requires_grad_(True)
    Y = bitmap_matmul(mask, X, recompute_plan=recompute)
    loss = (Y * Gt.float()).sum()
    loss.backward()
    A64, X64, G64 = bits.astype(np.float64), Xx.astype(np.float64), Gx.astype(np.float64)
    # forward
    assert _scaled_max(Y.detach().cpu().numpy() - A64 @ X64, A64 @ np.abs(X64)) <= TOL
    # dense PyTorch FP64 gradient of the same loss
    At = torch.from_numpy(A64).requires_grad_(True)
    Xd = torch.from_numpy(X64).requires_grad_(True)
    ((At @ Xd) * torch.from_numpy(G64)).sum().backward()
    dX_ref, dA_ref = Xd.grad.numpy(), At.grad.numpy()
    dX = X.grad.float().cpu().numpy()
    tolx = TOL if kind == "f32" else 1e-2  # dX is returned in X's dtype
    assert _scaled_max(dX - dX_ref, A64.T @ np.abs(G64)) <= tolx
    dA = mask.grad.cpu().numpy()
    assert np.all(dA[~bits] == 0)
    assert _scaled_max((dA - dA_ref)[bits], (np.abs(G64) @ np.abs(X64).T)[bits]) <= TOL
    # FP64 central differences on 64 random set coordinates (L is linear in A)
    ii, kk = np.nonzero(bits)
    pick = rng.choice(len(ii), 64, replace=False)
    h = 1e-3
    for t in pick:
        i, k = ii[t], kk[t]
        Ap = A64.copy(); Ap[i, k] += h
        Am = A64.copy(); Am[i, k] -= h
        fd = (_loss64(Ap, X64, G64) - _loss64(Am, X64, G64)) / (2 * h)
        assert abs(dA[i, k] - fd) <= 1e-3 * max(1.0, float(np.abs(G64[i]) @ np.abs(X64[k])))


@pytest.mark.slow
def test_config5_full_size_sample():
    cfg = W.config5()
    M, K, N = cfg["M"], cfg["K"], cfg["N"]
    words = cfg["words"]
    wd = words_dev(words)
    plan = ops.Plan(wd, K)
    X, G = bf16_dev(cfg["X"]), bf16_dev(cfg["G"])
    Xx, Gx = W.bf16_bits_to_f32(cfg["X"]), W.bf16_bits_to_f32(cfg["G"])
    Y = ops.spmm(wd, K, X, plan=plan)
    dX = ops.spmm_t(wd, M, K, G, plan=plan)
    dA = ops.sddmm(wd, M, K, G, X, plan=plan)
    assert capi.device_status() == 0
    rows = np.r_[0:64, 4032:4096]
    Ys = Y[torch.from_numpy(rows).cuda()].cpu().numpy()
    assert _scaled_max(Ys - O.spmm_f64(words[rows], K, Xx), O.spmm_abs_f64(words[rows], K, Xx)) <= TOL
    bits = W.unpack_bits(words, K)
    dXs = dX[torch.from_numpy(rows).cuda()].cpu().numpy().astype(np.float64)
    ref = bits[:, rows].T.astype(np.float64) @ Gx.astype(np.float64)
    assert _scaled_max(dXs - ref, bits[:, rows].T.astype(np.float64) @ np.abs(Gx).astype(np.float64)) <= TOL
    dAs = dA[torch.from_numpy(rows).cuda()].cpu().numpy()
    full = Gx[rows].astype(np.float64) @ Xx.astype(np.float64).T
    sc = np.abs(Gx[rows]).astype(np.float64) @ np.abs(Xx).astype(np.float64).T
    b = bits[rows]
    assert np.all(dAs[~b] == 0) and _scaled_max((dAs - full)[b], sc[b]) <= TOL
