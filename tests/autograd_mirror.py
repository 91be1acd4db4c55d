"""Verification harness only: torch.autograd.Function wrappers whose forward
and backward are the library's ops and hand-written adjoint kernels, so
torch's gradcheck can drive them.  Not part of the product."""
import numpy as np
import torch

import pdl_gb300 as P


def _pdl(t: torch.Tensor):
    return P.pdl(t.detach().cpu().numpy())


def _torch(x, like: torch.Tensor):
    return torch.from_numpy(np.ascontiguousarray(x.numpy())).to(like.dtype)


class SumOver(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a):
        ctx.save_for_backward(a)
        return _torch(P.sumover(_pdl(a)), a)

    @staticmethod
    def backward(ctx, g):
        (a,) = ctx.saved_tensors
        return _torch(P.sumover_bwd(_pdl(g), _pdl(a)), a)


class Average(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a):
        ctx.save_for_backward(a)
        return _torch(P.average(_pdl(a)), a)

    @staticmethod
    def backward(ctx, g):
        (a,) = ctx.saved_tensors
        return _torch(P.average_bwd(_pdl(g), _pdl(a)), a)


class Plus(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, b):
        ctx.save_for_backward(a, b)
        return _torch(P.plus(_pdl(a), _pdl(b)), a)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        ga, gb = P.plus_bwd(_pdl(g), _pdl(a), _pdl(b))
        return _torch(ga, a), _torch(gb, b)


class Mult(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, b):
        ctx.save_for_backward(a, b)
        return _torch(P.mult(_pdl(a), _pdl(b)), a)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        ga, gb = P.mult_bwd(_pdl(g), _pdl(a), _pdl(b))
        return _torch(ga, a), _torch(gb, b)


class MatMult(torch.autograd.Function):
    """numpy/torch order: a (..., h, t), b (..., t, w) -> c (..., h, w)."""

    @staticmethod
    def forward(ctx, a, b):
        ctx.save_for_backward(a, b)
        return _torch(P.matmult(_pdl(a), _pdl(b)), a)

    @staticmethod
    def backward(ctx, g):
        a, b = ctx.saved_tensors
        ga, gb = P.matmult_bwd(_pdl(g), _pdl(a), _pdl(b))
        return _torch(ga, a), _torch(gb, b)
