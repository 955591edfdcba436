"""ctypes binding of the C ABI declared in ``include/pypty_gb300.h``.

The CUDA library is mandatory: if it is missing or fails to load, ``lib()`` raises. There
is no CPU fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

PTY_OK = 0
PTY_ERR_INVALID = -1
PTY_ERR_UNSUPPORTED = -2
PTY_ERR_POSITION = -3
PTY_ERR_WORKSPACE = -4
PTY_ERR_CUDA = -5

ALGORITHMS = {"lsq_sqrt": 0, "ml": 1, "lsq": 2, "lsq_sqrt_2": 3}
# compressed-detector losses: pty_loss_and_direction_variants only
COMPRESSED_ALGORITHMS = {"lsq_compressed": 4, "gauss_compressed": 5, "poisson_compressed": 6}
RECON_TYPES = {"far_field": 0, "near_field": 1}
DFT_ENGINES = {"fp32_fft": 0, "bf16x3": 1, "bf16x6": 2}


class Problem(ctypes.Structure):
    """Mirror of ``pty_problem_t``."""
    _fields_ = [
        ("window", ctypes.c_int32), ("obj_ny", ctypes.c_int32), ("obj_nx", ctypes.c_int32),
        ("n_slices", ctypes.c_int32), ("n_obj_modes", ctypes.c_int32),
        ("n_probe_modes", ctypes.c_int32), ("n_positions", ctypes.c_int32),
        ("n_sequence", ctypes.c_int32), ("compute_batch", ctypes.c_int32),
        ("algorithm", ctypes.c_int32), ("step_obj", ctypes.c_int32),
        ("step_probe", ctypes.c_int32), ("step_pos", ctypes.c_int32),
        ("probe_shift", ctypes.c_int32), ("wavelength", ctypes.c_float),
        ("pixel_size_x", ctypes.c_float), ("pixel_size_y", ctypes.c_float),
        ("slice_distance", ctypes.c_float), ("edge_mult", ctypes.c_float),
        ("damping_cutoff", ctypes.c_float), ("smooth_rolloff", ctypes.c_float),
        ("loss_weight", ctypes.c_float), ("checkpoint_every", ctypes.c_int32),
        ("slice_distances", ctypes.c_void_p),
    ]


VSPACE_MAX_SEG = 7


class VSpace(ctypes.Structure):
    """Mirror of ``pty_vspace_t``: the optimizer's segments (object, probe, positions, tilts,
    static background, aberrations, beam current)."""
    _fields_ = [("n_seg", ctypes.c_int32), ("obj_seg", ctypes.c_int32),
                ("n", ctypes.c_int64 * VSPACE_MAX_SEG), ("weight", ctypes.c_double * VSPACE_MAX_SEG)]


class Variant(ctypes.Structure):
    """Mirror of ``pty_variant_t``: near field, compressed detectors, beam current, aberration
    plates, tilts, measured-data preprocessing, detector upsampling and the static background
    of ``pty_loss_and_direction_variants``."""
    _fields_ = [("recon_type", ctypes.c_int32), ("defocus", ctypes.c_float), ("cs", ctypes.c_float),
                ("tan_x", ctypes.c_float), ("tan_y", ctypes.c_float), ("n_masks", ctypes.c_int32),
                ("masks", ctypes.c_void_p), ("beam_current", ctypes.c_void_p),
                ("step_beam_current", ctypes.c_int32), ("beam_current_grad", ctypes.c_void_p),
                ("n_aberrations", ctypes.c_int32), ("n_aberration_sets", ctypes.c_int32),
                ("aberrations", ctypes.c_void_p), ("aberration_marker", ctypes.c_void_p),
                ("step_aberrations", ctypes.c_int32), ("aberrations_grad", ctypes.c_void_p),
                ("data_pad", ctypes.c_int32), ("use_padded_intensity", ctypes.c_int32),
                ("shift_y", ctypes.c_int32), ("shift_x", ctypes.c_int32), ("data_multiplier", ctypes.c_float),
                ("n_tilts", ctypes.c_int32), ("tilts_host", ctypes.c_void_p), ("tilt_mode", ctypes.c_int32),
                ("step_tilts", ctypes.c_int32), ("tilts_grad", ctypes.c_void_p),
                ("upsample_pattern", ctypes.c_int32), ("static_background", ctypes.c_void_p),
                ("step_static_background", ctypes.c_int32), ("static_background_grad", ctypes.c_void_p),
                ("defocus_per_position", ctypes.c_void_p), ("n_probe_scenarios", ctypes.c_int32),
                ("probe_marker", ctypes.c_void_p), ("exit_waves", ctypes.c_void_p),
                ("tilts_device", ctypes.c_void_p)]


class PtyError(RuntimeError):
    """A PTY_ERR_* status returned by the library."""

    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (what, _status_text(status), status))


_LIB = None
_VP = ctypes.c_void_p
_SZ = ctypes.c_size_t
_I32 = ctypes.c_int32
_I32P = ctypes.POINTER(ctypes.c_int32)
_F32P = ctypes.POINTER(ctypes.c_float)
_F64P = ctypes.POINTER(ctypes.c_double)
_PP = ctypes.POINTER(Problem)
_VS = ctypes.POINTER(VSpace)
_VARP = ctypes.POINTER(Variant)
_PPV = ctypes.POINTER(ctypes.c_void_p)
_F64 = ctypes.c_double
_F32 = ctypes.c_float
_I64 = ctypes.c_int64

SIGNATURES = {
    "pty_version": ([], ctypes.c_int),
    "pty_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "pty_workspace_bytes": ([_PP, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_loss_and_direction": ([_PP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _SZ, _VP],
                               ctypes.c_int),
    "pty_simulate_patterns": ([_PP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_fft2": ([_VP, _VP, _I32, _I32, _I32, _I32, _VP, _SZ, _VP], ctypes.c_int),
    "pty_fft2_workspace_bytes": ([_I32, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_split_workspace_bytes": ([_PP, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_forward": ([_PP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_backward": ([_PP, _VP, _VP, _VP, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_multislice_workspace_bytes": ([_I32] * 7 + [ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_multislice": ([_VP, _VP, _VP, ctypes.c_float] + [_I32] * 5 + [_VP, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_multislice_grads": ([_VP, _VP, _VP, _VP, ctypes.c_float, _VP, _VP] + [_I32] * 8 +
                             [_VP, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_scatteradd_workspace_bytes": ([_I32] * 5 + [ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_scatteradd": ([_VP, _I32, _I32, _I32, _VP, _I32, _I32, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_profile_begin": ([_I32], ctypes.c_int),
    "pty_profile_end": ([_F64P, _I32P, _I32], ctypes.c_int),
    "pty_kernel_name": ([_I32], ctypes.c_char_p),
    "pty_kernel_count": ([], ctypes.c_int),
    "pty_graph_cache_info": ([_I32P, _I32P, _I32P, ctypes.POINTER(_I64)], ctypes.c_int),
    "pty_fourier_clean_workspace_bytes": ([_I32, _I32, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_fourier_clean": ([_VP, _VP, _F64, _VP, _I32, _I32, _I64, _F32, _F32, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_fourier_clean_prepare": ([_I32, _I32, _F32, _F32, _VP, _VP, _SZ, _VP], ctypes.c_int),
    "pty_fourier_clean_apply": ([_VP, _VP, _F64, _VP, _I32, _I32, _I64, _VP, _SZ, _VP], ctypes.c_int),
    "pty_fft2_bf16x3_workspace_bytes": ([_I32, _I32, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_fft2_bf16x3": ([_VP, _VP, _I32, _I32, _I32, _VP, _SZ, _VP], ctypes.c_int),
    "pty_fft2_bf16x6_workspace_bytes": ([_I32, _I32, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_fft2_bf16x6": ([_VP, _VP, _I32, _I32, _I32, _VP, _SZ, _VP], ctypes.c_int),
    "pty_layered_workspace_bytes": ([_PP, _I32, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_loss_and_direction_layered": ([_PP, _I32] + [_VP] * 11 + [_SZ, _VP], ctypes.c_int),
    "pty_variants_workspace_bytes": ([_PP, _VARP, ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_loss_and_direction_variants": ([_PP, _VARP] + [_VP] * 11 + [_SZ, _VP], ctypes.c_int),
    "pty_nn_conv3x3": ([_VP, _VP, _VP, _VP] + [_I32] * 7 + [_VP], ctypes.c_int),
    "pty_nn_conv3x3_wgrad_workspace_floats": ([_I32] * 5 + [ctypes.POINTER(_I64)], ctypes.c_int),
    "pty_nn_conv3x3_wgrad": ([_VP] * 4 + [_I32] * 5 + [_VP, _VP], ctypes.c_int),
    "pty_nn_conv1x1": ([_VP] * 4 + [_I32] * 3 + [_I64, _VP], ctypes.c_int),
    "pty_nn_conv1x1_workspace_floats": ([_I32] * 3 + [_I64, ctypes.POINTER(_I64)], ctypes.c_int),
    "pty_nn_conv1x1_backward": ([_VP] * 6 + [_I32] * 3 + [_I64, _VP, _VP], ctypes.c_int),
    "pty_nn_relu_mask": ([_VP, _VP, _I64, _VP], ctypes.c_int),
    "pty_nn_add": ([_VP, _VP, _I64, _VP], ctypes.c_int),
    "pty_nn_avgpool2": ([_VP, _VP, _I64, _I32, _I32, _I32, _VP], ctypes.c_int),
    "pty_nn_upsample2": ([_VP, _VP] + [_I32] * 7 + [_VP], ctypes.c_int),
    "pty_nn_channel_copy": ([_VP, _VP] + [_I32] * 4 + [_I64, _I32, _VP], ctypes.c_int),
    "pty_nn_bilinear": ([_VP, _VP] + [_I32] * 7 + [_F32] * 4 + [_VP], ctypes.c_int),
    "pty_nn_mse": ([_VP, _VP, _VP, _VP, _I64, _VP], ctypes.c_int),
    "pty_nn_adam": ([_VP] * 4 + [_I64, _F32, _F32, _F32, _F32, _VP], ctypes.c_int),
    "pty_virtual_detectors": ([_VP, _I32, _I32, _F32, _VP, _VP], ctypes.c_int),
    "pty_atom_slices": ([_VP, _I32, _I32, _I32, _I32, _F32, _VP, _VP, _VP], ctypes.c_int),
    "pty_lbfgs_state_bytes": ([ctypes.POINTER(_SZ)], ctypes.c_int),
    "pty_lbfgs_reset": ([_VS, _VP, _VP], ctypes.c_int),
    "pty_lbfgs_first_direction": ([_VS, _PPV, _PPV, _VP, _VP], ctypes.c_int),
    "pty_lbfgs_steepest": ([_VS, _PPV, _PPV, _VP, _VP], ctypes.c_int),
    "pty_lbfgs_two_loop": ([_VS, _PPV, _PPV, _I32, _PPV, _PPV, _I32P, _VP, _VP], ctypes.c_int),
    "pty_lbfgs_dot": ([_VS, _PPV, _PPV, _I32, _VP, _VP], ctypes.c_int),
    "pty_lbfgs_axpy": ([_VS, _PPV, _PPV, _PPV, _F64, _VP], ctypes.c_int),
    "pty_lbfgs_accept": ([_VS, _F64, _PPV, _PPV, _PPV, _PPV, _PPV, _I32, _VP, _VP], ctypes.c_int),
    "pty_lbfgs_read": ([_VP, _F64P, _VP], ctypes.c_int),
    "pty_orthogonalize_modes": ([_VP, _I64, _I32, _VP], ctypes.c_int),
}


def _status_text(status: int) -> str:
    if _LIB is None:
        return "status %d" % status
    return _LIB.pty_status_string(status).decode()


def lib(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load ``libpypty_gb300.so`` (building it first only when asked)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.lib_path()
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise ImportError("pypty_gb300 CUDA library not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    cdll = ctypes.CDLL(path)
    for name, (argtypes, restype) in SIGNATURES.items():
        fn = getattr(cdll, name)
        fn.argtypes = argtypes
        fn.restype = restype
    _LIB = cdll
    return _LIB


def check(status: int, what: str) -> None:
    if status != PTY_OK:
        raise PtyError(status, what)


def split_workspace_bytes(problem: Problem) -> int:
    n = _SZ(0)
    check(lib().pty_split_workspace_bytes(ctypes.byref(problem), ctypes.byref(n)), "pty_split_workspace_bytes")
    return int(n.value)


def workspace_bytes(problem: Problem) -> int:
    n = _SZ(0)
    check(lib().pty_workspace_bytes(ctypes.byref(problem), ctypes.byref(n)), "pty_workspace_bytes")
    return int(n.value)


class LaunchProfiler:
    """Per-kernel device time and launch counts of the library's own kernels, measured with
    CUDA events on the launching stream (``pty_profile_begin`` / ``pty_profile_end``)."""

    def __init__(self, max_launches: int = 4096):
        self.max_launches = max_launches
        self.ms = {}
        self.launches = {}

    def __enter__(self):
        check(lib().pty_profile_begin(self.max_launches), "pty_profile_begin")
        return self

    def __exit__(self, *exc):
        n = lib().pty_kernel_count()
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int32 * n)()
        check(lib().pty_profile_end(ms, cnt, n), "pty_profile_end")
        for k in range(n):
            name = lib().pty_kernel_name(k).decode()
            self.ms[name] = float(ms[k])
            self.launches[name] = int(cnt[k])
        return False

    @property
    def total_launches(self) -> int:
        return sum(self.launches.values())
