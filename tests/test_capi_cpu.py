"""The C-ABI library loads, exports every declared entry point, and rejects bad problems on
the host before touching the GPU (no compute calls here: this file runs without a GPU)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from pypty_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.lib()


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(pty_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    assert "pty_loss_and_direction" in declared_symbols()


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_status_strings(lib):
    assert lib.pty_version() >= 100
    assert lib.pty_status_string(0) == b"ok"
    assert b"range" in lib.pty_status_string(_lib.PTY_ERR_POSITION)


def problem(**kw):
    p = _lib.Problem()
    d = dict(window=64, obj_ny=128, obj_nx=128, n_slices=2, n_obj_modes=1, n_probe_modes=2,
             n_positions=4, n_sequence=4, compute_batch=4, algorithm=0, step_obj=1, step_probe=1,
             step_pos=0, probe_shift=0, wavelength=0.0197, pixel_size_x=0.1, pixel_size_y=0.1,
             slice_distance=2.0, edge_mult=1.0, damping_cutoff=2 / 3, smooth_rolloff=0.0,
             loss_weight=1.0)
    d.update(kw)
    for k, v in d.items():
        setattr(p, k, v)
    return p


def test_workspace_size_grows_with_batch(lib):
    a = _lib.workspace_bytes(problem(compute_batch=2))
    b = _lib.workspace_bytes(problem(compute_batch=4))
    assert 0 < a < b


@pytest.mark.parametrize("kw,status", [
    (dict(window=96), _lib.PTY_ERR_UNSUPPORTED),
    (dict(n_probe_modes=9), _lib.PTY_ERR_UNSUPPORTED),
    (dict(algorithm=7), _lib.PTY_ERR_UNSUPPORTED),
    (dict(n_slices=0), _lib.PTY_ERR_INVALID),
    (dict(step_pos=1, probe_shift=0), _lib.PTY_ERR_INVALID),
])
def test_invalid_problems_rejected(lib, kw, status):
    n = ctypes.c_size_t(0)
    assert lib.pty_workspace_bytes(ctypes.byref(problem(**kw)), ctypes.byref(n)) == status


def test_empty_sequence_needs_no_workspace(lib):
    n = ctypes.c_size_t(123)
    assert lib.pty_workspace_bytes(ctypes.byref(problem(n_sequence=0)), ctypes.byref(n)) == _lib.PTY_OK
    assert n.value == 0
    # the other fields are still checked
    assert lib.pty_workspace_bytes(ctypes.byref(problem(n_sequence=0, window=96)),
                                   ctypes.byref(n)) == _lib.PTY_ERR_UNSUPPORTED
    assert lib.pty_workspace_bytes(ctypes.byref(problem(n_sequence=-1)), ctypes.byref(n)) == _lib.PTY_ERR_INVALID


def _call_with_positions(lib, pos, seq):
    p = problem(n_positions=pos.shape[0], n_sequence=seq.shape[0])
    corr = np.zeros(pos.shape, np.float32)
    fake = ctypes.c_void_p(16)   # never dereferenced: the host check fails first
    return lib.pty_loss_and_direction(ctypes.byref(p), fake, fake, pos.ctypes.data, corr.ctypes.data,
                                      seq.ctypes.data, fake, fake, fake, fake, fake, fake, 1 << 40, None)


def test_window_outside_object_is_rejected_on_host(lib):
    pos = np.array([[0, 0], [10, 10], [64, 0], [0, 65]], np.int32)   # (0, 65): 65 + 64 > 128
    assert _call_with_positions(lib, pos, np.arange(4, dtype=np.int32)) == _lib.PTY_ERR_POSITION
    pos = np.array([[0, 0], [10, 10], [-1, 0], [0, 0]], np.int32)
    assert _call_with_positions(lib, pos, np.arange(4, dtype=np.int32)) == _lib.PTY_ERR_POSITION


def test_sequence_out_of_range_is_rejected_on_host(lib):
    pos = np.zeros((4, 2), np.int32)
    assert _call_with_positions(lib, pos, np.array([0, 1, 2, 4], np.int32)) == _lib.PTY_ERR_POSITION
