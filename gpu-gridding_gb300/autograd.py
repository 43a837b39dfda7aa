"""torch.autograd binding of the gridder: forward = gridding kernel,
backward = the hand-written adjoint (degridding) kernel.

The forward map is grid = sum_i c~_i * (weight_i * vis_i) over each
visibility's footprint (reference oskar_grid_wproj.c:190-209).  For a real
loss L with dL/dgrid = r (re, im pairs):
    u_i            = sum_footprint conj(c~_i) r          (degridding kernel)
    dL/dvis_i      = weight_i * u_i                      (re, im pair)
    dL/dweight_i   = Re(conj(vis_i) u_i)
Used for gradient checks of the adjoint; u, v, w are not differentiated.
"""
from __future__ import annotations

import torch


class GridWproj(torch.autograd.Function):
    """grid = GridWproj.apply(vis, weight, uu, vv, ww, stack, plan,
    cell_size_rad, w_scale, grid_size) with vis [N, 2], weight [N], returns a
    new [G, G, 2] grid holding this call's contributions."""

    @staticmethod
    def forward(ctx, vis, weight, uu, vv, ww, stack, plan, cell_size_rad,
                w_scale, grid_size):
        from . import grid_wproj_device
        G = int(grid_size)
        grid = torch.zeros((G, G, 2), dtype=vis.dtype, device=vis.device)
        norm = torch.zeros(1, dtype=torch.float64, device=vis.device)
        skipped = torch.zeros(1, dtype=torch.int64, device=vis.device)
        grid_wproj_device(plan, stack, uu.contiguous(), vv.contiguous(),
                          ww.contiguous(), vis.contiguous(),
                          weight.contiguous(), cell_size_rad, w_scale, G,
                          grid, norm, skipped)
        ctx.save_for_backward(vis, weight, uu, vv, ww)
        ctx.stack, ctx.plan = stack, plan
        ctx.cell_size_rad, ctx.w_scale, ctx.grid_size = (cell_size_rad,
                                                         w_scale, G)
        return grid

    @staticmethod
    def backward(ctx, grad_grid):
        from . import degrid_wproj_device
        vis, weight, uu, vv, ww = ctx.saved_tensors
        u = torch.empty((vis.shape[0], 2), dtype=vis.dtype, device=vis.device)
        degrid_wproj_device(ctx.plan, ctx.stack, uu.contiguous(),
                            vv.contiguous(), ww.contiguous(),
                            ctx.cell_size_rad, ctx.w_scale, ctx.grid_size,
                            grad_grid.contiguous(), u)
        grad_vis = grad_weight = None
        if ctx.needs_input_grad[0]:
            grad_vis = weight[:, None] * u
        if ctx.needs_input_grad[1]:
            grad_weight = vis[:, 0] * u[:, 0] + vis[:, 1] * u[:, 1]
        return (grad_vis, grad_weight, None, None, None, None, None, None,
                None, None)
