"""Differentiable batched solve: x = A^{-1} b as a torch.autograd.Function.

Forward: magma_?gesv_batched (LU with partial pivoting and the solve, one
call).  The LU factors and pivots are kept for the backward pass, which is one
call of magma_?gesv_adjoint_batched:
    gb = A^{-T} gx      (transposed solve reusing the forward factors), and
    gA = -gb x^T        (fused rank-nrhs outer product).
No refactorisation happens in the backward pass.  FP64 and FP32 CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import lib as _L
from .batched import Queue, _check, _prefix, _vp, gesv_batched, ptr_array


class BatchedSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A: torch.Tensor, B: torch.Tensor):
        if A.dim() != 3 or B.dim() != 3 or A.shape[1] != A.shape[2] or B.shape[1] != A.shape[1]:
            raise ValueError("A must be (batch, n, n) and B (batch, n, nrhs)")
        if not (A.is_cuda and B.is_cuda) or A.dtype != B.dtype:
            raise ValueError("A and B must be CUDA tensors of one floating dtype")
        S = A.detach().transpose(1, 2).contiguous()     # column-major storage, becomes LU
        X = B.detach().transpose(1, 2).contiguous()     # becomes the solution
        ipiv, info = gesv_batched(S, X)
        ctx.save_for_backward(S, ipiv, X)
        ctx.mark_non_differentiable(info)
        return X.transpose(1, 2), info

    @staticmethod
    def backward(ctx, gX: torch.Tensor, _ginfo):
        S, ipiv, X = ctx.saved_tensors
        b, n, _ = S.shape
        nrhs = X.shape[1]
        G = gX.transpose(1, 2).contiguous()             # becomes gb = A^{-T} gx
        GA = torch.empty((b, n, n), dtype=S.dtype, device=S.device)   # storage of gA
        lib = _L.load()
        q = Queue.current(S.device)
        dS, dP, dX, dG, dGA = ptr_array(S), ptr_array(ipiv), ptr_array(X), ptr_array(G), \
            ptr_array(GA)
        rc = getattr(lib, f"magma_{_prefix(S)}gesv_adjoint_batched")(
            n, nrhs, _vp(dS), n, _vp(dP), _vp(dX), n, _vp(dG), n, _vp(dGA), n, b, q.handle)
        _check(rc, "magma_gesv_adjoint_batched")
        gA = GA.transpose(1, 2) if ctx.needs_input_grad[0] else None
        gB = G.transpose(1, 2) if ctx.needs_input_grad[1] else None
        return gA, gB


def solve(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """x = A^{-1} B for a batch, differentiable in A and B (float64 or float32)."""
    X, _info = BatchedSolve.apply(A, B)
    return X


def solve_with_info(A: torch.Tensor, B: torch.Tensor):
    """As solve(), also returning the per-matrix info (first zero pivot, 1-based)."""
    return BatchedSolve.apply(A, B)
