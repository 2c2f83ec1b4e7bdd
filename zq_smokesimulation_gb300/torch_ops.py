"""PyTorch wrapper of the reverse mode: a torch.autograd.Function whose
forward runs the smoke rollout with a control force and whose backward runs
the library's hand-written adjoint kernels (zqs_adjoint_* through the C ABI).

The core stays in the CUDA library; this module only moves device pointers
and orders the work on torch's current stream.

    ctl = SmokeControl(grid, initial_state, nsteps=64, checkpoint_every=8)
    F = torch.zeros(3, D, H, W, device="cuda", requires_grad=True)
    rho = ctl(F)                        # final density, (D, H, W)
    loss = ((rho - target) ** 2).sum()
    loss.backward()                     # F.grad from the adjoint kernels
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import capi


class SmokeControl:
    """A grid rolled out nsteps steps from a fixed initial state under a
    per-cell control force F of shape (3, D, H, W)."""

    def __init__(self, grid: capi.Grid, initial_state: dict, nsteps: int, checkpoint_every: int = 8):
        self.grid = grid
        self.init = {k: np.ascontiguousarray(initial_state[k], dtype=np.float32)
                     for k in ("u", "v", "w", "T", "rho")}
        self.nsteps = nsteps
        self.adj = capi.Adjoint(grid, nsteps, checkpoint_every)

    def reset(self):
        g = self.grid
        g.upload(capi.FIELD_U, self.init["u"])
        g.upload(capi.FIELD_V, self.init["v"])
        g.upload(capi.FIELD_W, self.init["w"])
        g.upload(capi.FIELD_TEMPERATURE, self.init["T"])
        g.upload(capi.FIELD_DENSITY, self.init["rho"])

    def __call__(self, F: torch.Tensor) -> torch.Tensor:
        return _Rollout.apply(F, self)


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, F: torch.Tensor, ctl: SmokeControl) -> torch.Tensor:
        g = ctl.grid
        if not F.is_cuda:
            raise ValueError("the control force must be a CUDA tensor")
        Fc = F.detach().to(torch.float32).contiguous()
        if Fc.numel() != 3 * g.W * g.H * g.D:
            raise ValueError("the control force must have shape (3, D, H, W)")
        ctl.reset()
        stream = torch.cuda.current_stream(F.device).cuda_stream
        ctl.adj.forward_device(Fc.data_ptr(), stream)
        rho = torch.empty((g.D, g.H, g.W), device=F.device, dtype=torch.float32)
        capi.check(g.lib.zqs_grid_download(g.h, capi.FIELD_DENSITY, C.c_void_p(rho.data_ptr()), 1,
                                           C.c_void_p(stream)), "zqs_grid_download")
        ctx.ctl = ctl
        ctx.shape = F.shape
        return rho

    @staticmethod
    def backward(ctx, grad_rho: torch.Tensor):
        ctl = ctx.ctl
        g = ctl.grid
        gr = grad_rho.detach().to(torch.float32).contiguous()
        out = torch.empty((3, g.D, g.H, g.W), device=gr.device, dtype=torch.float32)
        stream = torch.cuda.current_stream(gr.device).cuda_stream
        ctl.adj.backward_device(gr.data_ptr(), out.data_ptr(), stream)
        return out.reshape(ctx.shape), None
