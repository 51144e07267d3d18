"""torch.autograd interface of the batched chi2 (galario_gb300.batch).

``chi2_profile(intensity, params, dataset, Rmin, dR, dxy, nxy)`` returns the
(B,) chi2 of B profile models and is differentiable with respect to
``intensity`` (B, nr) and ``params`` (B, 4) = (inc, PA, dRA, dDec);
``chi2_image(images, params, dataset, dxy, origin)`` the same for B images
(B, nxy, nxy) and ``params`` (B, 3) = (PA, dRA, dDec).  The backward pass
re-runs the forward launches together with the hand-written adjoint kernels
(the spectrum is recomputed, not stored between the passes), so parametric
models built from torch operations (for example rings with radius, width and
flux) get their gradients by the chain rule.
"""
from __future__ import annotations

import torch

from .batch import Dataset, chi2_image_batch, chi2_profile_batch


class Chi2ProfileBatch(torch.autograd.Function):
    @staticmethod
    def forward(ctx, intensity, params, dataset, Rmin, dR, dxy, nxy):
        ctx.save_for_backward(intensity, params)
        ctx.geo = (dataset, Rmin, dR, dxy, nxy)
        return chi2_profile_batch(dataset, intensity.detach(), params.detach(), Rmin, dR, dxy, nxy, grad=False)

    @staticmethod
    def backward(ctx, g):
        intensity, params = ctx.saved_tensors
        dataset, Rmin, dR, dxy, nxy = ctx.geo
        _, gI, gp = chi2_profile_batch(dataset, intensity.detach(), params.detach(), Rmin, dR, dxy, nxy, grad=True)
        g = g.to(torch.float32)[:, None]
        return (gI * g).to(intensity.dtype), (gp * g).to(params.dtype), None, None, None, None, None


def chi2_profile(intensity, params, dataset: Dataset, Rmin, dR, dxy, nxy):
    """Differentiable batched chi2 (see module docstring)."""
    return Chi2ProfileBatch.apply(intensity, params, dataset, Rmin, dR, dxy, nxy)


class Chi2ImageBatch(torch.autograd.Function):
    @staticmethod
    def forward(ctx, images, params, dataset, dxy, origin):
        ctx.save_for_backward(images, params)
        ctx.geo = (dataset, dxy, origin)
        return chi2_image_batch(dataset, images.detach(), params.detach(), dxy, origin=origin, grad=False)

    @staticmethod
    def backward(ctx, g):
        images, params = ctx.saved_tensors
        dataset, dxy, origin = ctx.geo
        _, gI, gp = chi2_image_batch(dataset, images.detach(), params.detach(), dxy, origin=origin, grad=True)
        g = g.to(torch.float32)
        return ((gI * g[:, None, None]).to(images.dtype), (gp * g[:, None]).to(params.dtype), None, None, None)


def chi2_image(images, params, dataset: Dataset, dxy, origin="upper"):
    """Differentiable batched chi2 of images (see module docstring)."""
    return Chi2ImageBatch.apply(images, params, dataset, dxy, origin)
