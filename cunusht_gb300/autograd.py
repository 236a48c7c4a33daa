"""Differentiable lensing: gclm2lenmap as a torch.autograd.Function.

backward with respect to gclm is the adjoint lensing operator (nusht2d1 at the
deflected points, cunusht_nusht2d1) and with respect to the scaled lensing
potential the hand-written pointing-Jacobian VJP (cunusht_lensing_vjp_dlm).
The reference has no gradient path; its adjoint (lenmap2gclm,
cunusht/deflection/GPU_nufft_transformer.py:581-673) is what the gclm
gradient reuses.

Gradient convention: PyTorch's for a real loss of complex leaves,
grad = dL/dRe + i dL/dIm.  alm arrays store each m > 0 coefficient once for a
real field (the field depends on 2 Re(a_lm ...)), so the gradient is twice the
adjoint output for m > 0 and its real part for m = 0.
"""
from __future__ import annotations

import torch

from . import _lib
from .transformer import GPU_cufinufft_transformer, _stream, to_device


def _alm_weights(lmax: int, device) -> torch.Tensor:
    """1 for the m = 0 block (first lmax + 1 entries), 2 for m > 0."""
    n = (lmax + 1) * (lmax + 2) // 2
    w = torch.full((n,), 2.0, dtype=torch.float64, device=device)
    w[:lmax + 1] = 1.0
    return w


def _to_torch_grad(adj: torch.Tensor, lmax: int) -> torch.Tensor:
    w = _alm_weights(lmax, adj.device)
    g = adj * w
    g[..., :lmax + 1] = g[..., :lmax + 1].real.to(g.dtype)
    return g


def lensing_vjp_dlm(T: GPU_cufinufft_transformer, gclm: torch.Tensor, dlm_scaled: torch.Tensor,
                    grad_map: torch.Tensor) -> torch.Tensor:
    """Adjoint-convention gradient of <grad_map, gclm2lenmap(gclm, dlm)> with
    respect to dlm_scaled (spin 0)."""
    g = to_device(gclm, "gclm", torch.complex128).reshape(-1)
    d = to_device(dlm_scaled, "dlm_scaled", torch.complex128).reshape(-1)
    gm = to_device(grad_map, "grad_map", torch.float64).reshape(-1)
    out = torch.empty((T.nalm,), dtype=torch.complex128, device="cuda")
    _lib.check(T._lib.cunusht_lensing_vjp_dlm(T._plan, 0, g.data_ptr(), _lib.F64, d.data_ptr(), _lib.F64,
                                              gm.data_ptr(), out.data_ptr(), _stream()))
    # the pointing cache of T now holds stale state relative to this call
    T.dlm_scaled = None
    T.ptg = None
    return out


class LensingFunction(torch.autograd.Function):
    """lenmap = gclm2lenmap(gclm, dlm_scaled) with gradients for both inputs."""

    @staticmethod
    def forward(ctx, gclm, dlm_scaled, T, spin):
        T.dlm_scaled = None  # never reuse a pointing computed outside autograd
        out = T.gclm2lenmap(gclm.detach(), T.lmax, T.lmax, dlm_scaled=dlm_scaled.detach(), spin=spin, verbose=0)
        ctx.save_for_backward(gclm.detach(), dlm_scaled.detach())
        ctx.T = T
        ctx.spin = spin
        return out

    @staticmethod
    def backward(ctx, grad_out):
        gclm, dlm = ctx.saved_tensors
        T, spin = ctx.T, ctx.spin
        grad_g = grad_d = None
        g = grad_out.contiguous()
        if ctx.needs_input_grad[0]:
            adj = T.lenmap2gclm(g, dlm, None, T.lmax, T.lmax, spin=spin, verbose=0)
            grad_g = _to_torch_grad(adj, T.lmax).to(gclm.dtype).reshape(gclm.shape)
        if ctx.needs_input_grad[1]:
            if spin != 0:
                raise NotImplementedError("gradient with respect to the deflection: spin 0 only")
            adj = lensing_vjp_dlm(T, gclm, dlm, g)
            grad_d = _to_torch_grad(adj, T.lmax).to(dlm.dtype).reshape(dlm.shape)
        return grad_g, grad_d, None, None


def gclm2lenmap(T: GPU_cufinufft_transformer, gclm: torch.Tensor, dlm_scaled: torch.Tensor, spin: int = 0):
    """Differentiable lensed map (torch autograd) on the transformer's plan."""
    return LensingFunction.apply(gclm, dlm_scaled, T, spin)
