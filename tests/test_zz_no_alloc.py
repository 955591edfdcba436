"""pty_fft2_noalloc: the window FFT for callers that cannot allocate device memory.

Such callers (an application whose memory pool owns every device allocation, code running
during CUDA graph capture, allocation-free real-time loops) call pty_fft2_noalloc, which
keeps its twiddle tables in a fixed array inside the library instead of a workspace. This
test calls it through the C ABI and compares it with pty_fft2 (caller workspace) on
consecutive calls, so the second call runs on the array the first call left behind.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FFT_TOL = 2e-6   # relative L2, as for pty_fft2 against float64 NumPy


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_fft2_noalloc_matches_fft2_on_consecutive_calls():
    import torch
    from pypty_gb300 import _lib

    lib = _lib.lib()
    fn = lib.pty_fft2_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(42)
    calls = [(128, 0, 0), (128, 1, 1), (64, 0, 1), (64, 1, 0)]
    for W, inverse, shift in calls:
        x = torch.from_numpy((rng.normal(size=(3, W, W)) + 1j * rng.normal(size=(3, W, W)))
                             .astype(np.complex64)).to(dev)
        need = ctypes.c_size_t(0)
        assert lib.pty_fft2_workspace_bytes(W, ctypes.byref(need)) == 0
        ws = torch.empty(need.value, dtype=torch.uint8, device=dev)
        ref = torch.empty_like(x)
        assert lib.pty_fft2(x.data_ptr(), ref.data_ptr(), 3, W, inverse, shift, ws.data_ptr(), ws.numel(),
                            stream.cuda_stream) == 0
        out = torch.full_like(x, float("nan"))
        assert fn(x.data_ptr(), out.data_ptr(), 3, W, inverse, shift, stream.cuda_stream) == 0
        torch.cuda.synchronize(dev)
        assert _rel(out.cpu().numpy(), ref.cpu().numpy()) <= FFT_TOL


def test_fft2_noalloc_rejects_windows_beyond_its_scratch():
    import torch
    from pypty_gb300 import _lib
    lib = _lib.lib()
    fn = lib.pty_fft2_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    x = torch.zeros((1, 256, 256), dtype=torch.complex64, device="cuda")
    assert fn(x.data_ptr(), x.data_ptr(), 1, 256, 0, 0, None) == _lib.PTY_ERR_UNSUPPORTED
