"""Window FFT wrappers with the call surface of ``pypty/fft.py`` on the GPU path.

``fft2``, ``ifft2``, ``shift_fft2`` and ``ifft2_ishift`` transform two axes of equal length
64 or 128 (the probe window) with the library's shared-memory window FFT. NumPy input
gives NumPy output (through the device); CUDA tensors stay on the device.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import default_engine


def _run(arr, axes, inverse, shift):
    is_numpy = not isinstance(arr, torch.Tensor)
    t = torch.from_numpy(np.ascontiguousarray(arr)) if is_numpy else arr
    in_dtype = t.dtype
    eng = default_engine()
    t = t.to(device=eng.device, dtype=torch.complex64)
    a0, a1 = (ax % t.dim() for ax in axes)
    moved = torch.movedim(t, (a0, a1), (-2, -1)).contiguous()
    out = eng.fft2(moved, inverse=inverse, shift=shift)
    out = torch.movedim(out, (-2, -1), (a0, a1))
    if is_numpy:
        res = out.cpu().numpy()
        return res.astype(np.complex128) if in_dtype in (torch.complex128, torch.float64) else res
    return out.contiguous()


def fft2(arr, axes=(0, 1), overwrite_x=False, xp=None):
    """Unnormalised 2D DFT over ``axes`` (``pypty/fft.py:114``)."""
    return _run(arr, axes, False, False)


def ifft2(arr, axes=(0, 1), overwrite_x=False, xp=None):
    """2D inverse DFT scaled by 1/(n0*n1) over ``axes`` (``pypty/fft.py:136``)."""
    return _run(arr, axes, True, False)


def shift_fft2(arr, axes=(0, 1), overwrite_x=False, xp=None):
    """fftshift(fft2(arr)) over ``axes`` (``pypty/fft.py:91``)."""
    return _run(arr, axes, False, True)


def ifft2_ishift(arr, axes=(0, 1), overwrite_x=False, xp=None):
    """ifft2(ifftshift(arr)) over ``axes`` (``pypty/fft.py:158``)."""
    return _run(arr, axes, True, True)
