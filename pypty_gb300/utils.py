"""``fourier_clean`` and the Wolfe tests with the reference's signatures.

``fourier_clean`` replaces ``pypty.utils.fourier_clean`` (``pypty/utils.py:102-150``) for
2D, 3D and 4D arrays whose first two extents are powers of two in [64, 8192]: the band
limit runs in the library's strided FFT kernels (``pty_fourier_clean``). NumPy inputs give
NumPy outputs; CUDA tensors stay on the device. ``wolfe_1`` / ``wolfe_2`` are the scalar
conditions of ``pypty/utils.py:326-368``.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import default_engine
from .optim import fourier_clean_


def fourier_clean(array, cutoff=0.66, mask=None, rolloff=0, default_float=np.float32, xp=None):
    """Band-limit ``array`` over axes 0 and 1 (``pypty/utils.py:102-150``): radius
    0.5 * cutoff cycles per pixel with an optional cosine roll-off, or the given mask
    (fftshifted order). The cutoff / roll-off arithmetic is float32, as the reference's
    callers pass them (``pypty/iterative.py:147-149``)."""
    if cutoff is None and mask is None:
        return array
    if isinstance(array, torch.Tensor):
        t = array.to(torch.complex64).contiguous()
        out = fourier_clean_(t, cutoff, rolloff, mask=mask)
        return out.to(array.dtype) if array.dtype != torch.complex64 else out
    host = array.get() if hasattr(array, "get") else np.asarray(array)
    eng = default_engine()
    t = torch.from_numpy(np.ascontiguousarray(host.astype(np.complex64, copy=False))).to(eng.device)
    out = fourier_clean_(t, cutoff, rolloff, mask=mask, out=t)
    res = out.cpu().numpy()
    return res.astype(host.dtype, copy=False) if np.iscomplexobj(host) else res


def wolfe_1(value, new_value, d_value, step, wolfe_c1=0.5):
    """Sufficient decrease (``pypty/utils.py:326-348``)."""
    return new_value <= value + wolfe_c1 * step * d_value


def wolfe_2(d_value, new_d_value, wolfe_c2=0.9):
    """Curvature condition (``pypty/utils.py:350-368``)."""
    return -1 * new_d_value <= -1 * d_value * wolfe_c2
