"""Torch-tensor front end of the C ABI (device memory and streams from torch).

Names follow include/bsp.h; each docstring names the reference kernel the
call replaces.  Tensors must live on the current CUDA device; results are
produced on torch's current stream.
"""
import ctypes as C

import torch

from . import capi
from .capi import call

_DT = {torch.float32: capi.F32, torch.float16: capi.F16, torch.bfloat16: capi.BF16,
       torch.int8: capi.I8, torch.uint8: capi.U8}


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _rowmajor(t, name):
    if t.dim() != 2 or t.stride(1) != 1:
        raise ValueError("%s must be a 2-D tensor with unit column stride" % name)
    return t.stride(0)


def words_per_row(k):
    return (k + 31) // 32


def pack_rows(dense, bit_order=capi.LSB_FIRST, out=None):
    """dense [M, K] -> packed row masks int32 [M, ceil(K/32)] (uint32 bits).
    Replaces dense2bitmask (reference source/src/main.cu:591-628)."""
    ld = _rowmajor(dense, "dense")
    M, K = dense.shape
    if out is None:
        out = torch.empty((M, words_per_row(K)), dtype=torch.int32, device=dense.device)
    call("bsp_pack_rows", _p(dense), _DT[dense.dtype], M, K, ld, _p(out), bit_order, _stream())
    return out


def pack_cols(dense, bit_order=capi.LSB_FIRST, out=None):
    """dense [M, K] -> column masks [K, ceil(M/32)] (packed rows of the transpose)."""
    ld = _rowmajor(dense, "dense")
    M, K = dense.shape
    if out is None:
        out = torch.empty((K, words_per_row(M)), dtype=torch.int32, device=dense.device)
    call("bsp_pack_cols", _p(dense), _DT[dense.dtype], M, K, ld, _p(out), bit_order, _stream())
    return out


def transpose_bits(words, M, K, out=None):
    if out is None:
        out = torch.empty((K, words_per_row(M)), dtype=torch.int32, device=words.device)
    call("bsp_transpose_bits", _p(words), M, K, _p(out), _stream())
    return out


def unpack_rows(words, M, K, dtype=torch.float32, bit_order=capi.LSB_FIRST, out=None):
    """Packed masks -> dense 0/1 [M, K] (the scatter of group2dense for a full mask)."""
    if out is None:
        out = torch.empty((M, K), dtype=dtype, device=words.device)
    ld = _rowmajor(out, "out")
    call("bsp_unpack_rows", _p(words), M, K, _p(out), _DT[out.dtype], ld, bit_order, _stream())
    return out


def bitplanes(values, planes=8, bit_order=capi.LSB_FIRST, out=None):
    """uint8/int8 [M, K] -> packed bit planes [planes, M, ceil(K/32)].
    Replaces uint8_layout_trans (reference backup/layout_trans.cu:87-97)."""
    ld = _rowmajor(values, "values")
    M, K = values.shape
    if out is None:
        out = torch.empty((planes, M, words_per_row(K)), dtype=torch.int32, device=values.device)
    call("bsp_bitplanes", _p(values), M, K, ld, planes, _p(out), bit_order, _stream())
    return out


def group_rows(words, tile_rows, max_groups):
    """First-fit grouping of packed rows per (tile_rows × 32-column) tile.
    Replaces generate_groups_large (reference source/src/main.cu:50-247)."""
    M, Kw = words.shape
    T = ((M + tile_rows - 1) // tile_rows) * Kw
    dev = words.device
    out = dict(
        group_id=torch.empty((M, Kw), dtype=torch.int32, device=dev),
        group_mask=torch.empty((T, max_groups), dtype=torch.int32, device=dev),
        group_row=torch.empty((T, max_groups, 32), dtype=torch.int32, device=dev),
        spill_cnt=torch.empty(T, dtype=torch.int32, device=dev),
        spill_nnz=torch.empty(T, dtype=torch.int32, device=dev),
        spill_rows=torch.empty((T, tile_rows), dtype=torch.int32, device=dev),
        grouped_nnz=torch.empty(1, dtype=torch.int64, device=dev),
    )
    call("bsp_group_rows", _p(words), M, Kw, tile_rows, max_groups, _p(out["group_id"]),
         _p(out["group_mask"]), _p(out["group_row"]), _p(out["spill_cnt"]), _p(out["spill_nnz"]),
         _p(out["spill_rows"]), _p(out["grouped_nnz"]), _stream())
    return out


def group_to_dense(group_values, group_id, words, M, K, tile_rows, max_groups, out=None):
    """Replaces group2dense (reference source/src/main.cu:829-850)."""
    if out is None:
        out = torch.zeros((M, K), dtype=torch.float32, device=words.device)
    call("bsp_group_to_dense", _p(group_values), _p(group_id), _p(words), M, K, tile_rows,
         max_groups, _p(out), out.stride(0), _stream())
    return out


class Plan:
    """SpMM schedule for one A (similarity row grouping).  Owns device memory."""

    def __init__(self, words, K, mode=capi.PLAN_AUTO, signature_hashes=0, min_cluster_rows=0,
                 seed=0):
        self.M, Kw = words.shape
        self.K = K
        if Kw != words_per_row(K):
            raise ValueError("words has %d columns, expected ceil(K/32)=%d" % (Kw, words_per_row(K)))
        prm = capi.PlanParams(mode, signature_hashes, min_cluster_rows, seed)
        h = C.c_void_p()
        call("bsp_plan_create", _p(words), self.M, K, C.byref(prm), C.byref(h), _stream())
        self._h = h
        self._lib = capi.lib()

    @property
    def handle(self):
        return self._h

    def info(self):
        inf = capi.PlanInfo()
        call("bsp_plan_get_info", self._h, C.byref(inf))
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def workspace_bytes(self, N, preferred=True):
        """Workspace for spmm with this plan; ``preferred`` includes room for
        the tensor-core split of the reduction (bsp_spmm_workspace_preferred),
        else the minimum (bsp_spmm_workspace)."""
        n = C.c_size_t()
        call("bsp_spmm_workspace_preferred" if preferred else "bsp_spmm_workspace", self._h, N, C.byref(n))
        return n.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.bsp_plan_destroy(self._h)
            self._h = None

    def close_async(self):
        """Release the plan in stream order on the current stream (after the
        work already queued there), without waiting for the device."""
        if getattr(self, "_h", None):
            h, self._h = self._h, None
            call("bsp_plan_destroy_async", h, _stream())

    def __del__(self):
        self.close()


def spmm(words, K, B, plan=None, out=None, workspace=None):
    """C = A·B, FP32 output.  A: packed rows [M, ceil(K/32)], B: [K, N]
    float32/bfloat16/float16.  Replaces uint8_spmm_2d_1d / indexed_spmm
    (reference backup/layout_trans.cu:120-171)."""
    M = words.shape[0]
    ldb = _rowmajor(B, "B")
    if B.shape[0] != K:
        raise ValueError("B must have K rows")
    N = B.shape[1]
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device=B.device)
    ldc = _rowmajor(out, "out")
    h = plan.handle if plan is not None else None
    ws_ptr, ws_n = None, 0
    if plan is not None:
        # a caller's workspace is used if it holds the minimum; without one,
        # the preferred size (room for the tensor-core split) is allocated
        have = workspace.numel() * workspace.element_size() if workspace is not None else 0
        if workspace is None or have < plan.workspace_bytes(N, preferred=False):
            need = plan.workspace_bytes(N)
            workspace = torch.empty(max(need, 1), dtype=torch.uint8, device=B.device) if need else None
        if workspace is not None:
            ws_ptr, ws_n = _p(workspace), workspace.numel() * workspace.element_size()
    call("bsp_spmm", _p(words), M, K, _p(B), _DT[B.dtype], ldb, N, _p(out), ldc, h, ws_ptr, ws_n,
         _stream())
    return out


def spmm_t(words, M, K, G, plan=None, out=None, workspace=None):
    """dX = Aᵀ·G (FP32 [K, N]).  A: packed rows [M, ceil(K/32)], G: [M, N]."""
    ldg = _rowmajor(G, "G")
    N = G.shape[1]
    if out is None:
        out = torch.empty((K, N), dtype=torch.float32, device=G.device)
    n_min, n_pref = C.c_size_t(), C.c_size_t()
    call("bsp_spmm_t_workspace", M, K, C.byref(n_min))
    call("bsp_spmm_t_workspace_preferred", M, K, N, C.byref(n_pref))
    # a caller's workspace is used if it holds the minimum; else the preferred size
    if workspace is None or workspace.numel() * workspace.element_size() < n_min.value:
        workspace = torch.empty(n_pref.value, dtype=torch.uint8, device=G.device)
    call("bsp_spmm_t", _p(words), M, K, _p(G), _DT[G.dtype], ldg, N, _p(out), out.stride(0),
         plan.handle if plan is not None else None, _p(workspace),
         workspace.numel() * workspace.element_size(), _stream())
    return out


def sddmm(words, M, K, G, X, plan=None, out=None):
    """Straight-through mask gradient: dense [M, K] FP32 with (G·Xᵀ)[i, k] at
    A's set bits and 0 elsewhere.  G: [M, N], X: [K, N], same dtype."""
    ldg = _rowmajor(G, "G")
    ldx = _rowmajor(X, "X")
    if G.dtype != X.dtype:
        raise ValueError("G and X must have the same dtype")
    N = G.shape[1]
    if out is None:
        out = torch.empty((M, K), dtype=torch.float32, device=G.device)
    call("bsp_sddmm", _p(words), M, K, _p(G), ldg, _p(X), ldx, _DT[G.dtype], N, _p(out),
         out.stride(0), plan.handle if plan is not None else None, _stream())
    return out


def tune(words, K, B, plan, out=None, workspace=None):
    """Time every SpMM schedule for this plan and operands (bsp_tune), keep
    the fastest in the library's per-shape-bucket cache and return it as a
    dict (engine 1 = tensor cores, 2 = CUDA cores; the tensor-core tile form:
    K tiles per stage, B pre-tiled or by boxes, split-K; the prototype path
    and shape; ms).  ``out`` ends holding the product."""
    M = words.shape[0]
    ldb = _rowmajor(B, "B")
    N = B.shape[1]
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device=B.device)
    need = plan.workspace_bytes(N)
    if workspace is None or workspace.numel() * workspace.element_size() < need:
        workspace = torch.empty(max(need, 1), dtype=torch.uint8, device=B.device)
    best = capi.Schedule()
    call("bsp_tune", _p(words), M, K, _p(B), _DT[B.dtype], ldb, N, _p(out), out.stride(0), plan.handle,
         _p(workspace), workspace.numel() * workspace.element_size(), _stream(), C.byref(best))
    return {"engine": best.engine, "proto_path": best.proto_path, "proto_variant": best.proto_variant,
            "tc_stage_tiles": best.tc_stage_tiles, "tc_tiled_b": best.tc_tiled_b, "tc_split": best.tc_split,
            "ms": best.ms}


def symbolic_rows(a_words, K, b_words, N, out=None, plan=None, workspace=None):
    """Bit pattern of A·B for two bit matrices: row i of the result [M,
    ceil(N/32)] is the OR of B's row masks at A's set bits.  The symbolic
    half of pre_spgemm (reference source/src/transform.cuh:1028-1057);
    group_rows on the result is its output grouping.  With a prototype plan
    of A the rows come from their clusters' counts and delta lists (same
    result)."""
    M = a_words.shape[0]
    if b_words.shape[0] != K:
        raise ValueError("b_words must have K rows")
    if out is None:
        out = torch.empty((M, words_per_row(N)), dtype=torch.int32, device=a_words.device)
    if plan is not None:
        if workspace is None:
            workspace = _ws("bsp_symbolic_workspace", plan._h, N, device=a_words.device)
        call("bsp_symbolic_rows_planned", _p(a_words), M, K, _p(b_words), N, _p(out), plan._h, _p(workspace),
             workspace.numel(), _stream())
    else:
        call("bsp_symbolic_rows", _p(a_words), M, K, _p(b_words), N, _p(out), _stream())
    return out


def bitplane_spmm(planes, K, B, signed=True, out=None):
    """C = sum_b w_b (P_b B) for packed bit planes [n_planes, M, ceil(K/32)]
    (as ``bitplanes`` returns them), w_b = 2^b and -2^(n-1) for the top plane
    when ``signed``.  Replaces the bit-serial int8 product of
    spgemm_compute_1dthread_tcore_v3 (transform.cuh:2199-2246)."""
    n_planes, M, _ = planes.shape
    ldb = _rowmajor(B, "B")
    if B.shape[0] != K:
        raise ValueError("B must have K rows")
    N = B.shape[1]
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device=B.device)
    call("bsp_bitplane_spmm", _p(planes), n_planes, int(signed), M, K, _p(B), _DT[B.dtype], ldb, N,
         _p(out), out.stride(0), _stream())
    return out


def spmm_i8(A, B, out=None, workspace=None):
    """C = A·B for a dense int8 A [M, K]: bit planes in a workspace, then the
    signed bit-plane product (the reference's layout_trans + bit-serial path)."""
    lda = _rowmajor(A, "A")
    if A.dtype != torch.int8:
        raise ValueError("A must be int8")
    M, K = A.shape
    ldb = _rowmajor(B, "B")
    N = B.shape[1]
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device=B.device)
    need = C.c_size_t(0)
    call("bsp_spmm_i8_workspace", M, K, C.byref(need))
    if workspace is None or workspace.numel() * workspace.element_size() < need.value:
        workspace = torch.empty(need.value, dtype=torch.uint8, device=B.device)
    call("bsp_spmm_i8", _p(A), M, K, lda, _p(B), _DT[B.dtype], ldb, N, _p(out), out.stride(0),
         _p(workspace), workspace.numel() * workspace.element_size(), _stream())
    return out


def bitplanes_rows(values, planes=8, out=None):
    """uint8/int8 [M, K] -> bit planes side by side per row, [M, planes *
    ceil(K/32)] (a bitmap of planes * 32 * ceil(K/32) columns)."""
    ld = _rowmajor(values, "values")
    M, K = values.shape
    if out is None:
        out = torch.empty((M, planes * words_per_row(K)), dtype=torch.int32, device=values.device)
    call("bsp_bitplanes_rows", _p(values), M, K, ld, planes, _p(out), _stream())
    return out


def stack_planes_b(B, K, planes=8, signed=True, out=None):
    """[planes * 32 * ceil(K/32), N] blocks w_b * B (zero rows pad each block)."""
    ldb = _rowmajor(B, "B")
    N = B.shape[1]
    Kp = words_per_row(K) * 32
    if out is None:
        out = torch.empty((planes * Kp, N), dtype=B.dtype, device=B.device)
    call("bsp_stack_planes_b", _p(B), _DT[B.dtype], ldb, K, N, planes, int(signed), _p(out), out.stride(0),
         _stream())
    return out


class Int8Matrix:
    """An int8 matrix A [M, K] prepared for repeated products C = A·B: its 8
    bit planes side by side per row (a bitmap with 8·32·ceil(K/32) columns)
    and a plan of that bitmap.  ``matmul(B)`` stacks the plane-weighted
    copies of B and runs the planned bitmap SpMM, which takes the tensor
    cores for 16-bit B when the plan's cost model picks them — the
    reference's bit-serial int8 product (transform.cuh:2199-2246) with the
    2^b recombination folded into B."""

    def __init__(self, A, **plan_kw):
        if A.dtype != torch.int8 or A.dim() != 2:
            raise ValueError("A must be a 2-D int8 tensor")
        self.M, self.K = A.shape
        self.Kc = 8 * words_per_row(self.K) * 32
        self.words = bitplanes_rows(A.contiguous().view(torch.uint8), 8)
        self.plan = Plan(self.words, self.Kc, **plan_kw)

    def matmul(self, B, out=None, B_stacked=None):
        if B.shape[0] != self.K:
            raise ValueError("B must have K rows")
        Bs = stack_planes_b(B, self.K, 8, True, out=B_stacked)
        return spmm(self.words, self.Kc, Bs, plan=self.plan, out=out)

    def close(self):
        self.plan.close()


def _ws(fn, *args, device):
    need = C.c_size_t(0)
    call(fn, *args, C.byref(need))
    return torch.empty(max(need.value, 1), dtype=torch.uint8, device=device)


def rows_to_tiles8(words, K):
    """Packed rows [M, ceil(K/32)] -> the tSparse 8x8 bitmap tiles
    (reference coo2bmp_noTuple_d, source/src/main.cu:692-779): returns
    (bmp int64 [n], tile_row int32 [n], tile_col int32 [n], offset int32
    [n+1]); one host synchronisation reads n."""
    M = words.shape[0]
    dev = words.device
    T = ((M + 7) // 8) * ((K + 7) // 8)
    bmp = torch.empty(max(T, 1), dtype=torch.int64, device=dev)
    tr = torch.empty(max(T, 1), dtype=torch.int32, device=dev)
    tc = torch.empty(max(T, 1), dtype=torch.int32, device=dev)
    off = torch.empty(T + 1, dtype=torch.int32, device=dev)
    n = torch.empty(1, dtype=torch.int64, device=dev)
    ws = _ws("bsp_tiles8_workspace", M, K, device=dev)
    call("bsp_rows_to_tiles8", _p(words), M, K, _p(bmp), _p(tr), _p(tc), _p(off), _p(n), _p(ws),
         ws.numel(), _stream())
    k = int(n.item())
    return bmp[:k], tr[:k], tc[:k], off[: k + 1]


def tiles8_to_rows(bmp, tile_row, tile_col, M, K, out=None):
    """8x8 bitmap tiles -> packed rows [M, ceil(K/32)]."""
    if out is None:
        out = torch.empty((M, words_per_row(K)), dtype=torch.int32, device=bmp.device)
    call("bsp_tiles8_to_rows", _p(bmp), _p(tile_row), _p(tile_col), bmp.numel(), M, K, _p(out), _stream())
    return out


def csr_to_tiled(row_ptr, col_idx, M, K, tile_rows, tile_cols, values=None):
    """CSR -> tiled CSR of csr2tiledcsr (reference source/src/main.cu:499-588):
    returns (tile_nnz_acc [T+1], tiled_offset [T, tile_rows+1], tiled_col
    [nnz], tiled_values [nnz] or None)."""
    dev = row_ptr.device
    nnz = col_idx.numel()
    T = ((M + tile_rows - 1) // tile_rows) * ((K + tile_cols - 1) // tile_cols)
    acc = torch.empty(T + 1, dtype=torch.int32, device=dev)
    toff = torch.empty((T, tile_rows + 1), dtype=torch.int32, device=dev)
    tcol = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    tval = torch.empty(max(nnz, 1), dtype=values.dtype, device=dev) if values is not None else None
    ws = _ws("bsp_csr_to_tiled_workspace", M, K, nnz, tile_rows, tile_cols, device=dev)
    call("bsp_csr_to_tiled", _p(row_ptr), _p(col_idx), _p(values) if values is not None else None,
         values.element_size() if values is not None else 0, M, K, nnz, tile_rows, tile_cols, _p(acc), _p(toff),
         _p(tcol), _p(tval) if tval is not None else None, _p(ws), ws.numel(), _stream())
    return acc, toff, tcol[:nnz], (tval[:nnz] if tval is not None else None)


class Batch:
    """Many independent C_i = A_i·B_i (16-bit B, shared N) in one tensor-core
    launch: for N ≤ 128 a persistent kernel (a CTA per SM, 256-row items from
    a device work queue), otherwise a CTA per 256x256 item.  Runs of one
    batch must not overlap on the GPU (they share the queue and the C buffers).  ``problems``: list of (words, K, B, C) tensors; the
    tensors are referenced by the batch and must outlive it."""

    def __init__(self, problems):
        n = len(problems)
        if n == 0:
            raise ValueError("empty batch")
        N = problems[0][2].shape[1]
        dt = problems[0][2].dtype
        arr = (capi.Problem * n)()
        self._keep = []
        for i, (words, K, B, Cout) in enumerate(problems):
            if B.dtype != dt or B.shape[1] != N or Cout.shape[1] != N:
                raise ValueError("all problems of a batch share N and the B dtype")
            arr[i] = capi.Problem(words.data_ptr() if words.numel() else 0, words.shape[0], K,
                                  B.data_ptr() if B.numel() else 0, _rowmajor(B, "B"),
                                  Cout.data_ptr() if Cout.numel() else 0, _rowmajor(Cout, "C"))
            self._keep.append((words, B, Cout))
        h = C.c_void_p()
        call("bsp_batch_create", arr, n, N, _DT[dt], C.byref(h), _stream())
        self._h = h
        self._lib = capi.lib()

    def run(self):
        call("bsp_batched_spmm", self._h, _stream())

    def tune(self):
        """Time the persistent kernel's shapes on this batch (runs it four
        times per shape), keep the fastest for later runs; returns (shape,
        ms)."""
        shape, ms = C.c_int(), C.c_float()
        call("bsp_batch_tune", self._h, _stream(), C.byref(shape), C.byref(ms))
        return shape.value, ms.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.bsp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class BatchGrad:
    """Backward pass of many Y_i = A_i·X_i (16-bit X and G, shared N) in two
    tensor-core launches: dX_i = A_iᵀ·G_i and dA_i = (G_i·X_iᵀ) ⊙ A_i.
    ``problems``: list of (words, K, X, G, dX, dA) tensors, dX or dA may be
    None; the tensors are referenced by the batch and must outlive it.  Runs
    of one batch must not overlap on the GPU (they write dX and dA)."""

    def __init__(self, problems):
        n = len(problems)
        if n == 0:
            raise ValueError("empty batch")
        N = problems[0][2].shape[1]
        dt = problems[0][2].dtype
        arr = (capi.ProblemGrad * n)()
        self._keep = []
        ptr = lambda t: t.data_ptr() if t is not None and t.numel() else 0  # noqa: E731
        for i, (words, K, X, G, dX, dA) in enumerate(problems):
            if X.dtype != dt or G.dtype != dt or X.shape[1] != N or G.shape[1] != N:
                raise ValueError("all problems of a batch share N and the X / G dtype")
            arr[i] = capi.ProblemGrad(ptr(words), words.shape[0], K, ptr(X), _rowmajor(X, "X"), ptr(G),
                                      _rowmajor(G, "G"), ptr(dX), _rowmajor(dX, "dX") if dX is not None else 0,
                                      ptr(dA), _rowmajor(dA, "dA") if dA is not None else 0)
            self._keep.append((words, X, G, dX, dA))
        h = C.c_void_p()
        call("bsp_batch_grad_create", arr, n, N, _DT[dt], C.byref(h), _stream())
        self._h = h
        self._lib = capi.lib()

    def run(self):
        call("bsp_batched_spmm_grad", self._h, _stream())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.bsp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
