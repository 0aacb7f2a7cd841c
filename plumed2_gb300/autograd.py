"""torch.autograd binding of the COORDINATION CV.

    from plumed2_gb300.action import Coordination
    from plumed2_gb300.autograd import coordination

    act = Coordination("GROUPA=1-1000 SWITCH={RATIONAL R_0=0.3 D_MAX=1.0}", precision="mixed")
    s = coordination(act, pos, box, r0, d0)        # pos: (F, N, 3) float64 CUDA tensor
    V = bias(s); V.sum().backward()                # pos.grad, box.grad, r0.grad, d0.grad

The forward runs the s-only pair pass; the backward runs the library's
backward kernel (coord_backward_device), which returns dV/dx, dV/dh (box,
scaled coordinates held fixed) and dV/dR_0, dV/dD_0 in one pass over the
pairs of the forward's neighbour lists.  ``r0``/``d0`` are 0-d tensors holding
the action's own R_0 and D_0 (they carry the parameter gradients; their values
must equal those the action was created with).  Boxes are (F, 3, 3) and may
live on the CPU or the GPU (they are read on the host for the set-up).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def _boxes_host(box: torch.Tensor, n_frames: int) -> np.ndarray:
    b = box.detach().to("cpu", torch.float64).reshape(-1, 9).numpy()
    if b.shape[0] == 1 and n_frames > 1:
        b = np.repeat(b, n_frames, axis=0)
    return np.ascontiguousarray(b)


class CoordinationFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, box, r0, d0, action, step):
        if pos.dtype != torch.float64 or not pos.is_cuda:
            raise TypeError("positions must be a float64 CUDA tensor of shape (frames, slots, 3)")
        pos = pos.contiguous()
        F = pos.shape[0]
        boxes = _boxes_host(box, F)
        s = torch.empty(F, dtype=torch.float64, device=pos.device)
        stream = torch.cuda.current_stream(pos.device).cuda_stream
        action.forward_device(pos.data_ptr(), boxes, F, s.data_ptr(), 0, 0, step=step, flags=_lib.FLAG_NO_DERIV,
                              stream=stream)
        ctx.save_for_backward(pos)
        ctx.action = action
        ctx.boxes = boxes
        ctx.box_shape = box.shape
        ctx.box_device = box.device
        return s

    @staticmethod
    def backward(ctx, grad_s):
        (pos,) = ctx.saved_tensors
        F = pos.shape[0]
        g = grad_s.detach().to(torch.float64).contiguous()
        gpos = torch.empty_like(pos)
        gbox = torch.empty(F, 9, dtype=torch.float64, device=pos.device)
        gpar = torch.empty(F, 2, dtype=torch.float64, device=pos.device)
        stream = torch.cuda.current_stream(pos.device).cuda_stream
        ctx.action.backward_device(pos.data_ptr(), ctx.boxes, F, g.data_ptr(), gpos.data_ptr(), gbox.data_ptr(),
                                   gpar.data_ptr(), stream=stream)
        gb = gbox.reshape(F, 3, 3)
        if len(ctx.box_shape) == 2:
            gb = gb.sum(0)
        gb = gb.reshape(ctx.box_shape).to(ctx.box_device)
        return gpos, gb, gpar[:, 0].sum(), gpar[:, 1].sum(), None, None


def coordination(action, pos: torch.Tensor, box: torch.Tensor, r0: torch.Tensor | None = None,
                 d0: torch.Tensor | None = None, step: int = 0) -> torch.Tensor:
    """s per frame, differentiable in positions, box, R_0 and D_0."""
    dev = pos.device
    if r0 is None:
        r0 = torch.tensor(1.0 / action.switch_params()["invr0"], dtype=torch.float64, device=dev)
    if d0 is None:
        d0 = torch.tensor(action.switch_params()["d0"], dtype=torch.float64, device=dev)
    squeeze = pos.dim() == 2
    if squeeze:
        pos = pos.unsqueeze(0)
    s = CoordinationFunction.apply(pos, box, r0, d0, action, step)
    return s[0] if squeeze else s


class CoordinationNumbersFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, box, cns, step):
        if pos.dtype != torch.float64 or not pos.is_cuda:
            raise TypeError("positions must be a float64 CUDA tensor of shape (frames, slots, 3)")
        pos = pos.contiguous()
        F = pos.shape[0]
        boxes = _boxes_host(box, F)
        cn = torch.empty(F, pos.shape[1], dtype=torch.float64, device=pos.device)
        stream = torch.cuda.current_stream(pos.device).cuda_stream
        cns.forward_device(pos.data_ptr(), boxes, F, cn.data_ptr(), stream=stream, step=step)
        ctx.save_for_backward(pos)
        ctx.cns = cns
        ctx.boxes = boxes
        ctx.box_shape = box.shape
        ctx.box_device = box.device
        return cn

    @staticmethod
    def backward(ctx, grad_cn):
        (pos,) = ctx.saved_tensors
        F = pos.shape[0]
        g = grad_cn.detach().to(torch.float64).contiguous()
        gpos = torch.empty_like(pos)
        gbox = torch.empty(F, 9, dtype=torch.float64, device=pos.device)
        stream = torch.cuda.current_stream(pos.device).cuda_stream
        ctx.cns.backward_device(pos.data_ptr(), ctx.boxes, F, g.data_ptr(), gpos.data_ptr(), gbox.data_ptr(),
                                stream=stream)
        gb = gbox.reshape(F, 3, 3)
        if len(ctx.box_shape) == 2:
            gb = gb.sum(0)
        gb = gb.reshape(ctx.box_shape).to(ctx.box_device)
        return gpos, gb, None, None


def coordination_numbers(cns, pos: torch.Tensor, box: torch.Tensor, step: int = 0) -> torch.Tensor:
    """Per-slot coordination numbers (frames, slots) of a CoordinationNumbers
    action, differentiable in positions and box (one vector-Jacobian product
    over the forward's pairs)."""
    squeeze = pos.dim() == 2
    if squeeze:
        pos = pos.unsqueeze(0)
    cn = CoordinationNumbersFunction.apply(pos, box, cns, step)
    return cn[0] if squeeze else cn
