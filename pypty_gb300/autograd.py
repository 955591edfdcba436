"""The multislice loss as a differentiable torch function.

``multislice_loss(obj, probe, pos_correction, ...)`` returns the scalar loss of
``pypty.objective.loss_and_direction`` (``pypty/objective.py:47``) and differentiates it
with the library's own adjoint kernels: the forward call (``pty_forward``) runs the forward
multislice and the loss and keeps the wave stack on the device; ``backward`` runs the
adjoint multislice (``pty_backward``) only when a gradient is requested.

Gradient convention: the library returns the Wirtinger derivative dL/dz* (as the
reference does); torch's gradient of a real function of a complex tensor is 2 dL/dz*, so
``backward`` scales by 2. Position corrections are real: their gradient is dL/d(dy, dx).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .engine import Engine, Geometry, default_engine, make_problem


class _MultisliceLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, obj, probe, pos_correction, engine, positions, sequence, measured, options):
        need_obj, need_probe, need_pos = ctx.needs_input_grad[:3]
        corr = pos_correction.detach().cpu().numpy()
        geo = Geometry.make(positions, corr, sequence)
        W = probe.shape[0]
        prob = make_problem(W, tuple(obj.shape), probe.shape[2], geo, step_obj=need_obj, step_probe=need_probe,
                            step_pos=need_pos, **options)
        loss_sse, ws = engine.forward(prob, obj.detach().contiguous(), probe.detach().contiguous(), geo,
                                      measured)
        ctx.engine, ctx.problem, ctx.ws = engine, prob, ws
        ctx.pos_device = pos_correction.device
        return loss_sse[0].clone()

    @staticmethod
    def backward(ctx, grad_loss):
        need_obj, need_probe, need_pos = ctx.needs_input_grad[:3]
        if not (need_obj or need_probe or need_pos):
            return (None,) * 8
        _, og, pg, posg = ctx.engine.backward(ctx.problem, ctx.ws)
        ctx.ws = None
        g = grad_loss.to(torch.float32)
        d_obj = (2.0 * g) * og if need_obj else None
        d_probe = (2.0 * g) * pg if need_probe else None
        d_pos = (g * posg).to(ctx.pos_device) if need_pos else None
        return d_obj, d_probe, d_pos, None, None, None, None, None


def multislice_loss(obj: torch.Tensor, probe: torch.Tensor, pos_correction: torch.Tensor, positions,
                    measured: torch.Tensor, *, algorithm: str, wavelength: float, pixel_size_x: float,
                    pixel_size_y: float, slice_distance: float, sequence=None, edge_mult: float = 1.0,
                    damping_cutoff: float = 2 / 3, smooth_rolloff: float = 0.0, loss_weight: float = 1.0,
                    probe_shift: bool | None = None, engine: Engine | None = None) -> torch.Tensor:
    """Differentiable far-field multislice loss (a 0-d float64 tensor on the device).

    obj (Ny, Nx, Z, Mo) and probe (W, W, Mp) are complex64 CUDA tensors; pos_correction is a
    float32 (N, 2) tensor (host or device) of sub-pixel corrections; positions (N, 2) are the
    integer pixel positions; measured (N, W, W) float32 CUDA patterns in detector order.
    """
    engine = engine or default_engine(obj.device)
    if probe_shift is None:
        probe_shift = bool(torch.any(pos_correction != 0).item()) or pos_correction.requires_grad
    options = dict(algorithm=algorithm, wavelength=wavelength, pixel_size_x=pixel_size_x,
                   pixel_size_y=pixel_size_y, slice_distance=slice_distance, edge_mult=edge_mult,
                   damping_cutoff=damping_cutoff, smooth_rolloff=smooth_rolloff, loss_weight=loss_weight,
                   probe_shift=probe_shift)
    pos = np.asarray(positions.cpu().numpy() if isinstance(positions, torch.Tensor) else positions)
    seq = None if sequence is None else np.asarray(sequence)
    return _MultisliceLoss.apply(obj, probe, pos_correction, engine, pos, seq, measured, options)
