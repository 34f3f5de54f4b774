"""torch.autograd wrapper of the differentiable render: forward = spl_render
on device SoA inputs, backward = spl_render_backward.  A thin layer over the C
ABI; the gradient tests use it to drive the adjoint through torch.

Inputs: I (n,), colour (n, 3) -- palette value in column 0 for palette types,
RGB for colour-vector types --, world positions (n, 3), hsml (n,), all float32
on the renderer's device, the camera position (3,) float64 on the host
(centerpos, lookat and sky stay at the render context's values) and the
particle types as an int16 tensor on the device (not differentiated).
"""
from __future__ import annotations

import dataclasses

import numpy as np
import torch

from . import ParamFile, RenderContext, Renderer, _abi, frame_desc


class SplatRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, I, colour, pos, hsml, campos, renderer: Renderer, params: ParamFile,
                rc: RenderContext, ptype):
        rc2 = dataclasses.replace(rc, campos=campos.detach().cpu().numpy().astype(np.float64))
        keep: list = []
        desc = frame_desc(params, rc2, keep)
        soa = {"x": pos[:, 0].contiguous(), "y": pos[:, 1].contiguous(),
               "z": pos[:, 2].contiguous(), "r": hsml.contiguous(), "I": I.contiguous(),
               "cr": colour[:, 0].contiguous(), "cg": colour[:, 1].contiguous(),
               "cb": colour[:, 2].contiguous(), "type": ptype}
        pic = torch.empty((desc.xres, desc.yres, 3), dtype=torch.float32, device=I.device)
        renderer.set_stream(torch.cuda.current_stream(I.device).cuda_stream)
        renderer.set_differentiable(True)
        renderer.render_soa(desc, soa, pic, device=True)
        # the backward reads the forward's inputs through their device pointers
        ctx.keep = (soa, keep)
        ctx.renderer = renderer
        ctx.n = I.shape[0]
        return pic

    @staticmethod
    def backward(ctx, grad_pic):
        g = grad_pic.contiguous().to(torch.float32)
        dev = g.device
        out = {f: torch.zeros(ctx.n, dtype=torch.float32, device=dev) for f in _abi.GRAD_FIELDS}
        ctx.renderer.set_stream(torch.cuda.current_stream(dev).cuda_stream)
        res = ctx.renderer.backward(g, out, device=True)
        gcol = torch.stack([out["cr"], out["cg"], out["cb"]], dim=1)
        gpos = torch.stack([out["x"], out["y"], out["z"]], dim=1)
        gcam = torch.from_numpy(res["campos"])
        return out["I"], gcol, gpos, out["r"], gcam, None, None, None, None


def render(I, colour, pos, hsml, campos, renderer, params, rc, ptype):
    """Differentiable frame (x-major (xres, yres, 3) float32 image)."""
    return SplatRender.apply(I, colour, pos, hsml, campos, renderer, params, rc, ptype)
