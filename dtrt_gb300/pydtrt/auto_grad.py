"""ADLossFunc of the pydtrt API (reference pydtrt/auto_grad.py:21-75).

forward() renders the scene with the forward-mode GPU path tracer and keeps the nder
derivative images; backward() returns, per parameter, the sum over pixels of
dI/dtheta_i * dL/dI over an image pyramid (optionally clamping dL/dI to [-2, 2]).
"""
import math

import torch

from .. import dtrt


def downsample(x):
    """2x2 box filter with edge replication for odd sizes (auto_grad.py:11-16)."""
    if x.size(0) % 2 == 1:
        x = torch.cat((x, x[-1:, :]), dim=0)
    if x.size(1) % 2 == 1:
        x = torch.cat((x, x[:, -1:]), dim=1)
    return (x[0::2, 0::2, :] + x[1::2, 0::2, :] + x[0::2, 1::2, :] + x[1::2, 1::2, :]) * 0.25


class ADLossFunc(torch.autograd.Function):
    @staticmethod
    def forward(ctx, scene_manager, integrator, options, input, out_of_range=None, penalty_scale=None,
                pyramid_level=1, pyramid_scale=4.0, index_iter=-1, clamping=0):
        from .scene_renderer import render_scene
        n = scene_manager.nder
        if out_of_range is None:
            out_of_range = torch.zeros(n)
        if penalty_scale is None:
            penalty_scale = torch.ones(n)
        img = render_scene(integrator, options, *(scene_manager.args))
        if index_iter > -1:
            torch.save(img, "pt_iter%d.pt" % index_iter)
        ctx.save_for_backward(img[1:], torch.tensor([pyramid_level], dtype=torch.int),
                              torch.tensor([pyramid_scale], dtype=torch.float), out_of_range, penalty_scale,
                              torch.tensor([clamping], dtype=torch.int))
        return img[0]

    @staticmethod
    def backward(ctx, grad_input):
        derivs, lvl, pyramid_scale, out_of_range, penalty_scale, clamping = ctx.saved_tensors
        n = derivs.size(0)
        lvl = int(min(math.log(derivs.size(1), 2) + 1, math.log(derivs.size(2), 2) + 1, int(lvl)))
        ret = torch.zeros(n)
        cur = [derivs[k] for k in range(n)]
        g = grad_input
        for i in range(lvl):
            for k in range(n):
                if abs(out_of_range[k].item()) > 1e-4:
                    ret[k] = out_of_range[k] * penalty_scale[k]
                else:
                    gi = g
                    if int(clamping[0]) != 0:
                        gi = g.clone()
                        gi[g > 2.0] = 0.0
                        gi[g < -2.0] = 0.0
                    ret[k] += pow(float(pyramid_scale[0]), i) * (cur[k] * gi).sum()
                if i < lvl - 1:
                    cur[k] = downsample(cur[k])
            if i < lvl - 1:
                g = downsample(g)
        return (None, None, None, ret, None, None, None, None, None, None)
