"""``multislice``, ``multislice_grads`` and ``scatteradd`` with the reference's signatures.

Drop-ins for ``pypty.multislice_core`` (``pypty/multislice_core.py:9,85,206``) running on the
library's kernels (``pty_multislice``, ``pty_multislice_grads``, ``pty_scatteradd``). Arrays
use the reference layouts; NumPy inputs give NumPy outputs, CUDA tensors stay on the device.

Supported: one slice distance (``is_single_dist``), no tilts (``this_step_tilts == 0``),
window-shaped scatter indices (``masky = y_b + row index``, ``maskx = x_b + column index``),
windows of 64 or 128 px, Mp * Mo <= 8. Other combinations raise ``NotImplementedError``.
As in the reference, ``waves_multislice`` receives the conjugated wave stack and
``object_grad`` is accumulated in place; unlike the reference, ``dLoss_dP_out`` and
``waves_multislice`` are not overwritten by ``multislice_grads`` (their contents there are
scratch in the reference).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .engine import default_engine


def _unsupported(cond, what):
    if cond:
        raise NotImplementedError("pypty_gb300 multislice_core does not implement %s" % what)


def _dev(a, dtype):
    eng = default_engine()
    if isinstance(a, torch.Tensor):
        return a.to(device=eng.device, dtype=dtype).contiguous()
    if hasattr(a, "get"):
        a = a.get()
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=eng.device, dtype=dtype)


def _host(t, like):
    if isinstance(like, torch.Tensor):
        return t
    return t.cpu().numpy()


def _ws(nbytes):
    return default_engine().workspace(nbytes)


def _stream():
    return torch.cuda.current_stream(default_engine().device).cuda_stream


def _window_positions(masky, maskx, W):
    """(B, 2) window origins of window-shaped index arrays, or NotImplementedError."""
    my = np.asarray(masky.get() if hasattr(masky, "get") else masky)
    mx = np.asarray(maskx.get() if hasattr(maskx, "get") else maskx)
    my = my.reshape(my.shape[0], W, W) if my.ndim == 3 else my
    mx = mx.reshape(mx.shape[0], W, W) if mx.ndim == 3 else mx
    _unsupported(my.ndim != 3 or mx.ndim != 3 or my.shape[1:] != (W, W), "index arrays that are not windows")
    y0 = my[:, 0, 0].astype(np.int64)
    x0 = mx[:, 0, 0].astype(np.int64)
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    ok = np.array_equal(my, y0[:, None, None] + runy[None]) and np.array_equal(mx, x0[:, None, None] + runx[None])
    _unsupported(not ok, "index arrays that are not windows")
    return np.ascontiguousarray(np.stack([y0, x0], axis=1).astype(np.int32))


def multislice(full_probe, this_obj_chopped, num_slices, n_obj_modes, n_probe_modes, this_distances,
               edge_slice_thickness_multiplier, this_wavelength, q2, qx, qy, exclude_mask, is_single_dist,
               this_tan_x, this_tan_y, damping_cutoff_multislice, smooth_rolloff, master_propagator_phase_space,
               half_master_propagator_phase_space, mask_clean, waves_multislice, wave, tilt_mode,
               this_step_tilts, default_float, default_complex):
    """Forward multislice (``pypty/multislice_core.py:9-82``): returns (waves_multislice, wave)."""
    _unsupported(not is_single_dist or master_propagator_phase_space is None, "per-slice distances")
    _unsupported(bool(this_step_tilts), "tilt refinement")
    B, W = int(full_probe.shape[0]), int(full_probe.shape[1])
    Z, Mo, Mp = int(num_slices), int(n_obj_modes), int(n_probe_modes)
    probe_d = _dev(full_probe, torch.complex64)
    obj_d = _dev(this_obj_chopped, torch.complex64)
    prop = _dev(np.asarray(master_propagator_phase_space if not isinstance(master_propagator_phase_space,
                                                                             torch.Tensor)
                           else master_propagator_phase_space.cpu()).reshape(W, W), torch.complex64)
    dev = probe_d.device
    waves_d = torch.empty((B, W, W, Z, Mp, Mo), dtype=torch.complex64, device=dev)
    exit_d = torch.empty((B, W, W, Mp, Mo), dtype=torch.complex64, device=dev)
    n = ctypes.c_size_t(0)
    _lib.check(_lib.lib().pty_multislice_workspace_bytes(B, W, Z, Mp, Mo, 0, 0, ctypes.byref(n)),
               "pty_multislice_workspace_bytes")
    ws = _ws(int(n.value))
    _lib.check(_lib.lib().pty_multislice(probe_d.data_ptr(), obj_d.data_ptr(), prop.data_ptr(),
                                         float(edge_slice_thickness_multiplier), B, W, Z, Mp, Mo,
                                         waves_d.data_ptr(), exit_d.data_ptr(), ws.data_ptr(), ws.numel(),
                                         _stream()), "pty_multislice")
    if waves_multislice is not None:
        if isinstance(waves_multislice, torch.Tensor):
            waves_multislice[..., 0] = waves_d.to(waves_multislice.dtype)
        else:
            waves_multislice[..., 0] = waves_d.cpu().numpy()
        out_waves = waves_multislice
    else:
        out_waves = _host(waves_d, full_probe)[..., None]
    return out_waves, _host(exit_d, full_probe)


def multislice_grads(dLoss_dP_out, waves_multislice, this_obj_chopped, object_grad, tilts_grad, is_single_dist,
                     this_distances, edge_slice_thickness_multiplier, exclude_mask, this_wavelength, q2, qx,
                     this_tan_x, qy, this_tan_y, num_slices, n_obj_modes, tiltind, master_propagator_phase_space,
                     this_step_tilts, damping_cutoff_multislice, smooth_rolloff, tilt_mode, compute_batch,
                     mask_clean, this_step_probe, this_step_obj, this_step_pos_correction, masked_pixels_y,
                     masked_pixels_x, default_float, default_complex, helper_flag_4):
    """Adjoint multislice (``pypty/multislice_core.py:85-200``): returns
    (object_grad, interm_probe_grad, tilts_grad); object_grad is accumulated in place."""
    _unsupported(not is_single_dist or master_propagator_phase_space is None, "per-slice distances")
    _unsupported(bool(this_step_tilts), "tilt refinement")
    B, W = int(dLoss_dP_out.shape[0]), int(dLoss_dP_out.shape[1])
    Mp, Mo = int(dLoss_dP_out.shape[3]), int(dLoss_dP_out.shape[4])
    Z = int(num_slices)
    step_obj = bool(this_step_obj > 0)
    g_d = _dev(dLoss_dP_out, torch.complex64)
    obj_d = _dev(this_obj_chopped, torch.complex64)
    prop = _dev(np.asarray(master_propagator_phase_space if not isinstance(master_propagator_phase_space,
                                                                             torch.Tensor)
                           else master_propagator_phase_space.cpu()).reshape(W, W), torch.complex64)
    dev = g_d.device
    if step_obj:
        waves = waves_multislice[..., 0] if waves_multislice.ndim == 7 else waves_multislice
        waves_d = _dev(waves, torch.complex64)
        mask_d = _dev(np.asarray(mask_clean if not isinstance(mask_clean, torch.Tensor) else mask_clean.cpu())
                      .reshape(W, W), torch.float32)
        pos = _window_positions(masked_pixels_y, masked_pixels_x, W)
        og_d = _dev(object_grad, torch.complex64)
        Ny, Nx = int(object_grad.shape[0]), int(object_grad.shape[1])
    else:
        waves_d = mask_d = og_d = None
        pos = None
        Ny = Nx = 0
    pg_d = torch.empty((B, W, W, Mp), dtype=torch.complex64, device=dev) if helper_flag_4 else None
    n = ctypes.c_size_t(0)
    _lib.check(_lib.lib().pty_multislice_workspace_bytes(B, W, Z, Mp, Mo, Ny, Nx, ctypes.byref(n)),
               "pty_multislice_workspace_bytes")
    ws = _ws(int(n.value))
    ptr = (lambda t: t.data_ptr() if t is not None else None)
    _lib.check(_lib.lib().pty_multislice_grads(
        g_d.data_ptr(), ptr(waves_d), obj_d.data_ptr(), prop.data_ptr(), float(edge_slice_thickness_multiplier),
        ptr(mask_d), pos.ctypes.data if pos is not None else None, B, W, Z, Mp, Mo, Ny, Nx, int(step_obj),
        ptr(og_d), ptr(pg_d), ws.data_ptr(), ws.numel(), _stream()), "pty_multislice_grads")
    if step_obj:
        if isinstance(object_grad, torch.Tensor):
            object_grad.copy_(og_d.to(object_grad.dtype))
        else:
            object_grad[...] = og_d.cpu().numpy()
    interm = _host(pg_d, dLoss_dP_out) if pg_d is not None else None
    return object_grad, interm, tilts_grad


def scatteradd(full, masky, maskx, chop):
    """``full[masky, maskx] += chop`` (``pypty/multislice_core.py:206-230``), deterministic,
    for window-shaped index arrays; ``full`` is updated in place."""
    B, W = int(chop.shape[0]), int(chop.shape[1])
    Ny, Nx = int(full.shape[0]), int(full.shape[1])
    K = int(np.prod(full.shape[2:])) if len(full.shape) > 2 else 1
    _unsupported(tuple(chop.shape[3:]) != tuple(full.shape[2:]), "chop shapes that do not match full")
    pos = _window_positions(masky, maskx, W)
    full_d = _dev(full, torch.complex64)
    chop_d = _dev(chop, torch.complex64)
    n = ctypes.c_size_t(0)
    _lib.check(_lib.lib().pty_scatteradd_workspace_bytes(B, W, K, Ny, Nx, ctypes.byref(n)),
               "pty_scatteradd_workspace_bytes")
    ws = _ws(int(n.value))
    _lib.check(_lib.lib().pty_scatteradd(full_d.data_ptr(), Ny, Nx, K, pos.ctypes.data, B, W, chop_d.data_ptr(),
                                         ws.data_ptr(), ws.numel(), _stream()), "pty_scatteradd")
    if isinstance(full, torch.Tensor):
        full.copy_(full_d.to(full.dtype))
    else:
        full[...] = full_d.cpu().numpy()
    return None
