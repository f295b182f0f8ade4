"""torch.autograd.Function around the library's SVD and its adjoint kernel.

For validation of the hand-written adjoint only: forward runs the CUDA SVD
(FP32 arithmetic; a float64 input is decomposed in FP32 and the factors are
returned as float64), backward runs ddcsvd_svd_backward_{f32,f64}_device in
the dtype of the input.  Thin SVD of a batch (B, m, n) with m >= n:
returns U (B, m, n), S (B, n) ascending, V (B, n, n).
"""
from __future__ import annotations

import torch

from . import svd_backward_device, svd_batched_device


class SVD(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A):
        if A.dim() != 3 or A.shape[1] < A.shape[2]:
            raise ValueError("expected a batch (B, m, n) with m >= n")
        outs = svd_batched_device([a.float() for a in A.unbind(0)])
        U = torch.stack([o[1] for o in outs]).to(A.dtype)
        S = torch.stack([o[0] for o in outs]).to(A.dtype)
        V = torch.stack([o[2] for o in outs]).to(A.dtype)
        ctx.save_for_backward(U, S, V)
        return U, S, V

    @staticmethod
    def backward(ctx, gU, gS, gV):
        U, S, V = ctx.saved_tensors
        gA = svd_backward_device(U.contiguous(), S.contiguous(), V.contiguous(),
                                 None if gU is None else gU.contiguous(),
                                 None if gS is None else gS.contiguous(),
                                 None if gV is None else gV.contiguous())
        return gA


def svd(A):
    """Differentiable thin SVD (validation wrapper): (U, S ascending, V)."""
    return SVD.apply(A)
