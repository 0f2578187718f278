"""Differentiable bitmap SpMM: a thin torch.autograd.Function over the C ABI.

    Y = A · X        A: M×K 0/1 mask, X: K×N (FP32 / BF16 / FP16), Y FP32

Backward (hand-written, no autograd tracing of the kernels):

* dX = Aᵀ · dY           — ``bsp_spmm_t``: on the tensor cores the bit tiles
  of Aᵀ are read straight from A's packed rows, no transposed copy;
* dA = (dY · Xᵀ) ⊙ A     — ``bsp_sddmm``: the straight-through mask
  gradient, sampled only at A's set bits (0 elsewhere).

In the precision form dY is stored in X's 16-bit type before both products
(the forward output stays FP32); FP32 X keeps FP32 everywhere.  The mask is
packed to 1 bit per element for the saved state.  The similarity plan of A
(row grouping, tile occupancy) is kept for backward, or rebuilt there when
``recompute_plan=True`` (it then holds no device memory between the passes).
"""
import torch

from . import ops


class BitmapMatmul(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mask, X, plan, recompute_plan):
        if mask.dim() != 2 or X.dim() != 2 or mask.shape[1] != X.shape[0]:
            raise ValueError("mask must be M x K and X K x N")
        M, K = mask.shape
        words = ops.pack_rows(mask.contiguous())
        if plan is None:
            plan = ops.Plan(words, K)
        Xc = X.contiguous()
        Y = ops.spmm(words, K, Xc, plan=plan)
        ctx.save_for_backward(words, Xc)
        ctx.shape = (M, K)
        ctx.plan = None if recompute_plan else plan
        ctx.mask_dtype = mask.dtype
        return Y

    @staticmethod
    def backward(ctx, dY):
        words, X = ctx.saved_tensors
        M, K = ctx.shape
        plan = ctx.plan if ctx.plan is not None else ops.Plan(words, K)
        G = dY.contiguous().to(X.dtype)
        dmask = dX = None
        if ctx.needs_input_grad[1]:
            dX = ops.spmm_t(words, M, K, G, plan=plan).to(X.dtype)
        if ctx.needs_input_grad[0]:
            dA = ops.sddmm(words, M, K, G, X, plan=plan)
            dmask = dA if ctx.mask_dtype == torch.float32 else dA.to(ctx.mask_dtype)
        return dmask, dX, None, None


def bitmap_matmul(mask, X, plan=None, recompute_plan=False):
    """Y = mask · X with the hand-written backward above.  ``mask`` is a dense
    M×K tensor whose nonzeros are the set bits (bool or floating point; a
    floating mask with requires_grad receives the straight-through gradient);
    ``plan`` optionally reuses an ``ops.Plan`` of the packed mask."""
    return BitmapMatmul.apply(mask, X, plan, recompute_plan)
