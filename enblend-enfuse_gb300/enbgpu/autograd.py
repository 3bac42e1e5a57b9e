"""A thin torch.autograd.Function over enb_fuse_grad, for gradient checks.

The forward calls the C ABI's adjoint entry point, which returns the loss and
all gradients in one pass; the backward hands the stored gradients back,
scaled by the incoming gradient.  Only the loss is differentiable here (the
entry point computes dL/d(parameters), not a general vector-Jacobian
product of the fused image).
"""
from __future__ import annotations

from typing import Sequence

import torch

from . import Context, enfuse_params


class FuseLoss(torch.autograd.Function):
    """loss = mean((enfuse(images; theta, logits) - target)^2).

    Inputs: logits (K, H, W) float32 CUDA tensor, theta (5,) float64 tensor
    (exposure optimum, exposure width, exposure / saturation / contrast
    weights); non-differentiable: the context, the images, the target and the
    other weighting options."""

    @staticmethod
    def forward(fctx, logits, theta, ctx: Context, images: Sequence[torch.Tensor], target, options: dict):
        t = [float(v) for v in theta.detach().cpu().tolist()]
        prm = enfuse_params(exposure_optimum=t[0], exposure_width=t[1], exposure_weight=t[2], saturation_weight=t[3],
                            contrast_weight=t[4], float_range=options.get("float_range", 1.0),
                            exposure_weight_function=options.get("exposure_weight_function", "gaussian"),
                            contrast_window_size=options.get("contrast_window_size", 5), entropy_weight=0.0)
        lg = [x.contiguous() for x in logits.float()]
        gl = [torch.zeros_like(x) for x in lg]
        r = ctx.fuse_grad(list(images), target, params=prm, logits=lg, grad_logits=gl, levels=options.get("levels", 0))
        fctx.save_for_backward(torch.stack(gl), torch.tensor(
            [r["d_exp_optimum"], r["d_exp_width"], r["d_w_exposure"], r["d_w_saturation"], r["d_w_contrast"]],
            dtype=torch.float64))
        return torch.tensor(r["loss"], dtype=torch.float64)

    @staticmethod
    def backward(fctx, grad):
        g_logits, g_theta = fctx.saved_tensors
        return (g_logits * grad.to(g_logits.device, g_logits.dtype), g_theta * grad.to(g_theta.dtype),
                None, None, None, None)
