"""Device-resident driver of the C ABI: workspace, pinned staging and torch tensors.

PyTorch supplies device memory, streams and pinned host memory; every arithmetic step of
the path runs in the library's own CUDA kernels (``pypty_gb300/csrc``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib


@dataclass
class Geometry:
    """Scan geometry in host memory: the reference's integer positions, sub-pixel
    corrections and processing sequence (``pypty/utils.py:1742-1746``)."""
    positions: np.ndarray       # (N, 2) int32 [y, x]
    pos_correction: np.ndarray  # (N, 2) float32 [dy, dx]
    sequence: np.ndarray        # (n,) int32

    @staticmethod
    def make(positions, pos_correction, sequence=None) -> "Geometry":
        pos = np.ascontiguousarray(np.asarray(positions), dtype=np.int32)
        corr = np.ascontiguousarray(np.asarray(pos_correction), dtype=np.float32)
        if sequence is None:
            sequence = np.arange(pos.shape[0])
        seq = np.ascontiguousarray(np.asarray(sequence), dtype=np.int32)
        return Geometry(pos, corr, seq)

    def probe_shift(self, step_pos: bool) -> bool:
        """``probe_shift_flag`` of ``pypty/objective.py:347``."""
        return bool(np.sum(self.pos_correction.astype(np.float64) ** 2) != 0.0) or bool(step_pos)


def make_problem(W, obj_shape, n_probe_modes, geometry: Geometry, *, algorithm, wavelength,
                 pixel_size_x, pixel_size_y, slice_distance, edge_mult=1.0,
                 damping_cutoff=2 / 3, smooth_rolloff=0.0, loss_weight=1.0, compute_batch=None,
                 step_obj=True, step_probe=True, step_pos=False, probe_shift=None,
                 checkpoint_every=1, slice_distances=None) -> _lib.Problem:
    """The C-ABI problem description. ``slice_distances``: the reference's ``this_distances``
    when it has more than one entry (step z from slice z to z + 1 uses entry z,
    ``multislice_core.py:69-74``); None or one entry: ``slice_distance`` for every step."""
    ny, nx, nz, mo = obj_shape
    if isinstance(algorithm, str):
        codes = dict(_lib.ALGORITHMS, **_lib.COMPRESSED_ALGORITHMS)
        if algorithm not in codes:
            raise NotImplementedError("loss %r is not implemented on the GPU path" % algorithm)
        algorithm = codes[algorithm]
    if damping_cutoff is None:
        damping_cutoff = 2.0
    if damping_cutoff < 0:
        damping_cutoff = 2 / 3
    n = geometry.positions.shape[0]
    ns = geometry.sequence.shape[0]
    if probe_shift is None:
        probe_shift = geometry.probe_shift(step_pos)
    p = _lib.Problem()
    p.window, p.obj_ny, p.obj_nx, p.n_slices, p.n_obj_modes = W, ny, nx, nz, mo
    p.n_probe_modes, p.n_positions, p.n_sequence = n_probe_modes, n, ns
    p.compute_batch = int(compute_batch if compute_batch else ns)
    p.algorithm = int(algorithm)
    p.step_obj, p.step_probe, p.step_pos = int(bool(step_obj)), int(bool(step_probe)), int(bool(step_pos))
    p.probe_shift = int(bool(probe_shift))
    p.wavelength, p.pixel_size_x, p.pixel_size_y = wavelength, pixel_size_x, pixel_size_y
    p.slice_distance, p.edge_mult = slice_distance, edge_mult
    p.damping_cutoff, p.smooth_rolloff, p.loss_weight = damping_cutoff, smooth_rolloff, loss_weight
    p.checkpoint_every = int(checkpoint_every)
    p.slice_distances = None
    if slice_distances is not None:
        d = np.asarray(slice_distances, dtype=np.float32).reshape(-1)
        if d.shape[0] > 1 and nz > 1:
            if d.shape[0] < nz - 1:   # the reference indexes this_distances[z] for z < Z - 1
                raise ValueError("slice_distances needs n_slices - 1 = %d entries, got %d" % (nz - 1, d.shape[0]))
            d = np.ascontiguousarray(d[:nz - 1])
            p._slice_distances = d    # keeps the host array the struct points to alive
            p.slice_distances = d.ctypes.data
    return p


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


class Engine:
    """Workspace and staging buffers for repeated calls on one CUDA device."""

    def __init__(self, device=None):
        _lib.lib()
        self.device = torch.device(device if device is not None else "cuda")
        self._ws = None
        self._aux = {}
        self._aux_events = {}
        # two page-locked geometry buffers used in turn, each with the event of the call that
        # last read it: the host fills one while the GPU may still run the previous call
        self._stages = [None, None]
        self._stage_events = [None, None]
        self._stage_i = 0

    # ---------------------------------------------------------------- buffers
    def workspace(self, nbytes: int) -> torch.Tensor:
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = None
            self._ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
        return self._ws

    def aux(self, key: str, nbytes: int) -> torch.Tensor:
        """A device buffer of at least nbytes kept per key (small tables, optimizer state),
        separate from the loss-and-gradient workspace."""
        buf = self._aux.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = self._aux[key] = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
        return buf

    def _ordered_aux(self, key: str, nbytes: int, stream):
        """aux(key) for a call on `stream`, ordered after the previous call that used the same
        buffer (possibly on another stream); returns (buffer, mark) -- call mark() after the
        launch so that the next user waits for it."""
        buf = self.aux(key, nbytes)
        ev = self._aux_events.get(key)
        if ev is not None:
            stream.wait_event(ev)

        def mark():
            e = self._aux_events.get(key)
            if e is None:
                e = self._aux_events[key] = torch.cuda.Event()
            e.record(stream)
        return buf, mark

    def _staging(self, geo: Geometry, stream):
        """Page-locked copies of the geometry (the C ABI uploads them asynchronously). The call
        is also ordered on `stream` after the previous call (which may have run on another stream):
        the workspace is shared."""
        need = geo.positions.nbytes + geo.pos_correction.nbytes + geo.sequence.nbytes + 64
        self._stage_i ^= 1
        i = self._stage_i
        if self._stage_events[i ^ 1] is not None:
            stream.wait_event(self._stage_events[i ^ 1])
        if self._stage_events[i] is not None:
            self._stage_events[i].synchronize()     # the call before last has read this buffer
        if self._stages[i] is None or self._stages[i].numel() < need:
            self._stages[i] = torch.empty(need, dtype=torch.uint8, pin_memory=True)
        stage = self._stages[i]
        buf = stage.numpy()
        o = 0
        ptrs = []
        for arr in (geo.positions, geo.pos_correction, geo.sequence):
            n = arr.nbytes
            buf[o:o + n] = arr.view(np.uint8).reshape(-1)
            ptrs.append(stage.data_ptr() + o)
            o += (n + 15) // 16 * 16
        return ptrs

    def _mark_staging(self, stream):
        i = self._stage_i
        if self._stage_events[i] is None:
            self._stage_events[i] = torch.cuda.Event()
        self._stage_events[i].record(stream)

    # ---------------------------------------------------------------- calls
    def loss_and_direction(self, problem: _lib.Problem, obj: torch.Tensor, probe: torch.Tensor,
                           geo: Geometry, measured: torch.Tensor, out=None, stream=None,
                           pos_correction: torch.Tensor | None = None):
        """Run the fused path. obj (Ny,Nx,Z,Mo) complex64, probe (W,W,Mp) complex64 and
        measured (N,W,W) float32 on the device. Returns (loss_sse float64[2], object_grad,
        probe_grad, pos_grad) device tensors (loss_sse = [loss * loss_weight, sse]).
        pos_correction: optional (N, 2) float32 CUDA tensor used instead of the geometry's
        host corrections (the optimizer's device-resident trial positions)."""
        stream = stream or torch.cuda.current_stream(self.device)
        self._check_inputs(problem, obj, probe, measured)
        if out is None:
            out = (torch.empty(2, dtype=torch.float64, device=self.device),
                   torch.empty_like(obj), torch.empty_like(probe),
                   torch.empty((problem.n_positions, 2), dtype=torch.float32, device=self.device))
        loss_sse, og, pg, posg = out
        ws = self.workspace(_lib.workspace_bytes(problem))
        pp, pc, ps = self._staging(geo, stream)
        if pos_correction is not None:
            if (not pos_correction.is_cuda or pos_correction.dtype != torch.float32
                    or tuple(pos_correction.shape) != (problem.n_positions, 2)
                    or not pos_correction.is_contiguous()):
                raise ValueError("pos_correction must be a contiguous (N, 2) float32 CUDA tensor")
            pc = pos_correction.data_ptr()
        st = _lib.lib().pty_loss_and_direction(
            ctypes.byref(problem), _ptr(obj), _ptr(probe), pp, pc, ps, _ptr(measured),
            _ptr(loss_sse), _ptr(og), _ptr(pg), _ptr(posg), _ptr(ws), ws.numel(), stream.cuda_stream)
        self._mark_staging(stream)
        _lib.check(st, "pty_loss_and_direction")
        return loss_sse, og, pg, posg

    def loss_and_direction_layered(self, problem: _lib.Problem, obj: torch.Tensor, probe: torch.Tensor,
                                   geo: Geometry, measured: torch.Tensor, engine: str = "bf16x3", stream=None):
        """loss_and_direction with every window DFT on `engine` ("fp32_fft" or "bf16x3",
        ``pty_loss_and_direction_layered``): the precision sweep. Same outputs as
        ``loss_and_direction``."""
        stream = stream or torch.cuda.current_stream(self.device)
        self._check_inputs(problem, obj, probe, measured)
        eid = _lib.DFT_ENGINES[engine]
        n = ctypes.c_size_t(0)
        _lib.check(_lib.lib().pty_layered_workspace_bytes(ctypes.byref(problem), eid, ctypes.byref(n)),
                   "pty_layered_workspace_bytes")
        ws = self.workspace(int(n.value))
        out = (torch.empty(2, dtype=torch.float64, device=self.device), torch.empty_like(obj),
               torch.empty_like(probe), torch.zeros((problem.n_positions, 2), dtype=torch.float32, device=self.device))
        loss_sse, og, pg, posg = out
        pp, pc, ps = self._staging(geo, stream)
        st = _lib.lib().pty_loss_and_direction_layered(
            ctypes.byref(problem), eid, _ptr(obj), _ptr(probe), pp, pc, ps, _ptr(measured), _ptr(loss_sse),
            _ptr(og), _ptr(pg), _ptr(posg), _ptr(ws), ws.numel(), stream.cuda_stream)
        self._mark_staging(stream)
        _lib.check(st, "pty_loss_and_direction_layered")
        return loss_sse, og, pg, posg

    def loss_and_direction_variants(self, problem: _lib.Problem, obj: torch.Tensor, probe: torch.Tensor,
                                    geo: Geometry, measured: torch.Tensor, *, recon_type: str = "far_field",
                                    defocus: float = 0.0, cs: float = 0.0, tan_x: float = 0.0, tan_y: float = 0.0,
                                    masks: torch.Tensor | None = None, beam_current: torch.Tensor | None = None,
                                    step_beam_current: bool = False, aberrations: torch.Tensor | None = None,
                                    aberration_marker: torch.Tensor | None = None, step_aberrations: bool = False,
                                    data_pad: int = 0, use_padded_intensity: bool = True,
                                    data_shift_vector=(0, 0), data_multiplier: float = 1.0,
                                    tilts=None, tilt_mode: int = 0, step_tilts: bool = False,
                                    upsample_pattern: int = 1, static_background: torch.Tensor | None = None,
                                    step_static_background: bool = False,
                                    defocus_per_position: torch.Tensor | None = None,
                                    probe_marker: torch.Tensor | None = None,
                                    exit_waves: torch.Tensor | None = None,
                                    stream=None, pos_correction: torch.Tensor | None = None):
        """loss_and_direction with the near-field, compressed-detector, beam-current,
        aberration-plate and inside-tilt branches (``pty_loss_and_direction_variants``).

        measured is (n_positions, m, m) float32 (device memory, or pinned host memory read in
        place) with m = S / u - 2 (data_pad // u if use_padded_intensity else 0), S the pattern
        side after the data_pad crop (W with use_padded_intensity, else W - 2 data_pad) and
        u = upsample_pattern; or (n_positions, n_masks) for the compressed algorithms;
        data_pad / use_padded_intensity / data_shift_vector / data_multiplier are the
        reference's per-batch measured-data preprocessing, applied on the fly; upsample_pattern
        sums the model pattern over u x u blocks before the loss; static_background (W, W)
        float32 adds its square (band-limited) to every pattern, with step_static_background
        its gradient is returned; defocus_per_position (n_positions,) float32: near-field
        defocus of every position instead of ``defocus``; probe_marker (n_positions,) int with a
        4D probe (W, W, Mp, S): every position's probe scenario (the probe gradient is then
        (W, W, Mp, S) too); exit_waves (n_sequence, Mp, Mo, W, W) complex64 CUDA tensor: filled
        with every position's exit wave; tilts
        (n_tilts, 6) host array or CUDA tensor (the reference's tilt array plus its correction;
        one row or one per position) with tilt_mode 0-4 and step_tilts; masks (n_masks, W, W) float32 in pattern order; beam_current
        (n_positions,) float32; aberrations (n_sets, n_abs) float32 with aberration_marker
        (n_positions,) int32; pos_correction as in ``loss_and_direction``. Returns (loss_sse,
        object_grad, probe_grad, pos_grad, beam_current_grad or None, aberrations_grad or
        None, tilts_grad or None, static_background_grad or None)."""
        stream = stream or torch.cuda.current_stream(self.device)
        compressed = problem.algorithm in _lib.COMPRESSED_ALGORITHMS.values()
        n_scen = int(probe.shape[3]) if probe_marker is not None and probe.dim() == 4 else 1
        self._check_inputs(problem, obj, probe, None, n_scen)
        up = max(int(upsample_pattern), 1)
        side = problem.window if use_padded_intensity else problem.window - 2 * int(data_pad)
        wm = side // up - 2 * (int(data_pad) // up if use_padded_intensity else 0)
        want = (problem.n_positions, masks.shape[0]) if compressed else (problem.n_positions, wm, wm)
        if tuple(measured.shape) != want or measured.dtype != torch.float32 or not _readable(measured) \
                or not measured.is_contiguous():
            raise ValueError("measured must be a contiguous float32 CUDA or pinned host tensor of shape %s"
                             % (want,))
        if recon_type not in _lib.RECON_TYPES:
            raise NotImplementedError("recon_type %r" % recon_type)
        keep = []

        def dev(t, dtype):
            if t is None:
                return None
            t = t.to(device=self.device, dtype=dtype).contiguous()
            keep.append(t)
            return t

        if aberrations is not None:
            mk = np.asarray(aberration_marker.cpu() if torch.is_tensor(aberration_marker) else aberration_marker)
            if mk.shape != (problem.n_positions,) or mk.min() < 0 or mk.max() >= aberrations.shape[0]:
                raise ValueError("aberration_marker must hold one set index in [0, %d) per position"
                                 % aberrations.shape[0])
        masks_d = dev(masks, torch.float32)
        bc_d = dev(beam_current, torch.float32)
        ab_d = dev(aberrations, torch.float32)
        mk_d = dev(aberration_marker, torch.int32)
        bc_grad = torch.zeros(problem.n_positions, dtype=torch.float32, device=self.device) \
            if bc_d is not None and step_beam_current else None
        ab_grad = torch.zeros(tuple(ab_d.shape), dtype=torch.float32, device=self.device) \
            if ab_d is not None and step_aberrations else None
        pm_d = None
        if n_scen > 1:
            pm = np.asarray(probe_marker.cpu() if torch.is_tensor(probe_marker) else probe_marker)
            if pm.shape != (problem.n_positions,) or pm.min() < 0 or pm.max() >= n_scen:
                raise ValueError("probe_marker must hold one scenario index in [0, %d) per position" % n_scen)
            pm_d = dev(probe_marker, torch.int32)
        if exit_waves is not None:
            want_e = (problem.n_sequence, problem.n_probe_modes, problem.n_obj_modes, problem.window, problem.window)
            if (tuple(exit_waves.shape) != want_e or exit_waves.dtype != torch.complex64 or not exit_waves.is_cuda
                    or not exit_waves.is_contiguous()):
                raise ValueError("exit_waves must be a contiguous complex64 CUDA tensor of shape %s" % (want_e,))
        dfp_d = dev(defocus_per_position, torch.float32)
        if dfp_d is not None and tuple(dfp_d.shape) != (problem.n_positions,):
            raise ValueError("defocus_per_position must hold one defocus per position")
        sb_d = dev(static_background, torch.float32)
        if sb_d is not None and tuple(sb_d.shape) != (problem.window, problem.window):
            raise ValueError("static_background must be (W, W)")
        sb_grad = torch.zeros(tuple(sb_d.shape), dtype=torch.float32, device=self.device) \
            if sb_d is not None and step_static_background else None
        tilts_h = None
        tilts_d = None
        tilts_grad = None
        if tilts is not None:
            if torch.is_tensor(tilts) and tilts.is_cuda:
                # device rows (an optimizer's trial tilts): read in place, no host round trip
                tilts_d = dev(tilts.reshape(-1, 6), torch.float32)
                n_rows = int(tilts_d.shape[0])
            else:
                tilts_h = np.ascontiguousarray(np.asarray(tilts.cpu() if torch.is_tensor(tilts) else tilts,
                                                          dtype=np.float32).reshape(-1, 6))
                n_rows = int(tilts_h.shape[0])
            if n_rows not in (1, problem.n_positions):
                raise ValueError("tilts must have one row or one row per position")
            if step_tilts:
                tilts_grad = torch.zeros((n_rows, 6), dtype=torch.float32, device=self.device)
        v = _lib.Variant(recon_type=_lib.RECON_TYPES[recon_type], defocus=float(defocus), cs=float(cs),
                         tan_x=float(tan_x), tan_y=float(tan_y),
                         n_masks=0 if masks_d is None else int(masks_d.shape[0]),
                         masks=None if masks_d is None else masks_d.data_ptr(),
                         beam_current=None if bc_d is None else bc_d.data_ptr(),
                         step_beam_current=int(bc_grad is not None),
                         beam_current_grad=None if bc_grad is None else bc_grad.data_ptr(),
                         n_aberrations=0 if ab_d is None else int(ab_d.shape[1]),
                         n_aberration_sets=0 if ab_d is None else int(ab_d.shape[0]),
                         aberrations=None if ab_d is None else ab_d.data_ptr(),
                         aberration_marker=None if mk_d is None else mk_d.data_ptr(),
                         step_aberrations=int(ab_grad is not None),
                         aberrations_grad=None if ab_grad is None else ab_grad.data_ptr(),
                         data_pad=int(data_pad), use_padded_intensity=int(bool(use_padded_intensity)),
                         shift_y=int(data_shift_vector[0]), shift_x=int(data_shift_vector[1]),
                         data_multiplier=float(data_multiplier),
                         n_tilts=0 if tilts is None else n_rows,
                         tilts_host=None if tilts_h is None else tilts_h.ctypes.data,
                         tilts_device=None if tilts_d is None else tilts_d.data_ptr(),
                         tilt_mode=int(tilt_mode), step_tilts=int(tilts_grad is not None),
                         tilts_grad=None if tilts_grad is None else tilts_grad.data_ptr(),
                         upsample_pattern=up,
                         static_background=None if sb_d is None else sb_d.data_ptr(),
                         step_static_background=int(sb_grad is not None),
                         static_background_grad=None if sb_grad is None else sb_grad.data_ptr(),
                         defocus_per_position=None if dfp_d is None else dfp_d.data_ptr(),
                         n_probe_scenarios=n_scen, probe_marker=None if pm_d is None else pm_d.data_ptr(),
                         exit_waves=None if exit_waves is None else exit_waves.data_ptr())
        n = ctypes.c_size_t(0)
        _lib.check(_lib.lib().pty_variants_workspace_bytes(ctypes.byref(problem), ctypes.byref(v), ctypes.byref(n)),
                   "pty_variants_workspace_bytes")
        ws = self.workspace(int(n.value))
        loss_sse = torch.empty(2, dtype=torch.float64, device=self.device)
        og, pg = torch.empty_like(obj), torch.empty_like(probe)
        posg = torch.zeros((problem.n_positions, 2), dtype=torch.float32, device=self.device)
        pp, pc, ps = self._staging(geo, stream)
        if pos_correction is not None:
            if (not pos_correction.is_cuda or pos_correction.dtype != torch.float32
                    or tuple(pos_correction.shape) != (problem.n_positions, 2)
                    or not pos_correction.is_contiguous()):
                raise ValueError("pos_correction must be a contiguous (N, 2) float32 CUDA tensor")
            pc = pos_correction.data_ptr()
        st = _lib.lib().pty_loss_and_direction_variants(
            ctypes.byref(problem), ctypes.byref(v), _ptr(obj), _ptr(probe), pp, pc, ps, _ptr(measured),
            _ptr(loss_sse), _ptr(og), _ptr(pg), _ptr(posg), _ptr(ws), ws.numel(), stream.cuda_stream)
        self._mark_staging(stream)
        for t in keep:
            t.record_stream(stream)
        _lib.check(st, "pty_loss_and_direction_variants")
        return loss_sse, og, pg, posg, bc_grad, ab_grad, tilts_grad, sb_grad

    def forward(self, problem: _lib.Problem, obj: torch.Tensor, probe: torch.Tensor, geo: Geometry,
                measured: torch.Tensor, stream=None):
        """Forward half (pty_forward): returns (loss_sse, workspace). The workspace holds the
        wave stack and dL/d(exit wave) of every position until `backward` consumes it."""
        stream = stream or torch.cuda.current_stream(self.device)
        self._check_inputs(problem, obj, probe, measured)
        ws = torch.empty(max(_lib.split_workspace_bytes(problem), 256), dtype=torch.uint8, device=self.device)
        loss_sse = torch.empty(2, dtype=torch.float64, device=self.device)
        pp, pc, ps = self._staging(geo, stream)
        st = _lib.lib().pty_forward(ctypes.byref(problem), _ptr(obj), _ptr(probe), pp, pc, ps, _ptr(measured),
                                    _ptr(loss_sse), _ptr(ws), ws.numel(), stream.cuda_stream)
        self._mark_staging(stream)
        _lib.check(st, "pty_forward")
        return loss_sse, ws

    def backward(self, problem: _lib.Problem, ws: torch.Tensor, stream=None):
        """Adjoint half (pty_backward) on the workspace of `forward`: returns (loss_sse,
        object_grad, probe_grad, pos_grad) with the shapes of loss_and_direction."""
        stream = stream or torch.cuda.current_stream(self.device)
        W = problem.window
        loss_sse = torch.empty(2, dtype=torch.float64, device=self.device)
        og = torch.empty((problem.obj_ny, problem.obj_nx, problem.n_slices, problem.n_obj_modes),
                         dtype=torch.complex64, device=self.device)
        pg = torch.empty((W, W, problem.n_probe_modes), dtype=torch.complex64, device=self.device)
        posg = torch.empty((problem.n_positions, 2), dtype=torch.float32, device=self.device)
        st = _lib.lib().pty_backward(ctypes.byref(problem), _ptr(loss_sse), _ptr(og), _ptr(pg), _ptr(posg),
                                     _ptr(ws), ws.numel(), stream.cuda_stream)
        _lib.check(st, "pty_backward")
        return loss_sse, og, pg, posg

    def simulate(self, problem: _lib.Problem, obj: torch.Tensor, probe: torch.Tensor, geo: Geometry,
                 out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """Mean-over-modes far-field patterns (n_sequence, W, W) float32, detector order."""
        stream = stream or torch.cuda.current_stream(self.device)
        self._check_inputs(problem, obj, probe, None)
        W = problem.window
        if out is None:
            out = torch.empty((problem.n_sequence, W, W), dtype=torch.float32, device=self.device)
        ws = self.workspace(_lib.workspace_bytes(problem))
        pp, pc, ps = self._staging(geo, stream)
        st = _lib.lib().pty_simulate_patterns(ctypes.byref(problem), _ptr(obj), _ptr(probe), pp, pc, ps,
                                              _ptr(out), _ptr(ws), ws.numel(), stream.cuda_stream)
        self._mark_staging(stream)
        _lib.check(st, "pty_simulate_patterns")
        return out

    def fft2(self, x: torch.Tensor, inverse: bool = False, shift: bool = False, out=None, stream=None):
        """Batched 2D FFT over the last two axes of a (..., W, W) complex64 device tensor."""
        stream = stream or torch.cuda.current_stream(self.device)
        if x.dtype != torch.complex64 or not x.is_cuda:
            raise TypeError("fft2 needs a complex64 CUDA tensor")
        W = x.shape[-1]
        if x.shape[-2] != W:
            raise ValueError("fft2 needs square windows")
        x = x.contiguous()
        out = torch.empty_like(x) if out is None else out
        n = ctypes.c_size_t(0)
        _lib.check(_lib.lib().pty_fft2_workspace_bytes(W, ctypes.byref(n)), "pty_fft2_workspace_bytes")
        # its own buffer (not the loss-and-gradient workspace), ordered after its last user
        ws, mark = self._ordered_aux("fft2", int(n.value), stream)
        batch = x.numel() // (W * W)
        st = _lib.lib().pty_fft2(_ptr(x), _ptr(out), batch, W, int(inverse), int(shift), _ptr(ws),
                                 ws.numel(), stream.cuda_stream)
        mark()
        _lib.check(st, "pty_fft2")
        return out

    def fft2_bf16x3(self, x: torch.Tensor, inverse: bool = False, out=None, stream=None, terms: int = 2):
        """Batched 2D DFT over the last two axes of a (..., W, W) complex64 device tensor on the
        tensor cores in BF16x3 split precision (``pty_fft2_bf16x3``; W = 64, 128, 256); with
        terms=3 in BF16x6 (``pty_fft2_bf16x6``)."""
        stream = stream or torch.cuda.current_stream(self.device)
        if x.dtype != torch.complex64 or not x.is_cuda:
            raise TypeError("fft2_bf16x3 needs a complex64 CUDA tensor")
        W = x.shape[-1]
        if x.shape[-2] != W:
            raise ValueError("fft2_bf16x3 needs square windows")
        x = x.contiguous()
        out = torch.empty_like(x) if out is None else out
        batch = x.numel() // (W * W)
        n = ctypes.c_size_t(0)
        name = "pty_fft2_bf16x3" if terms == 2 else "pty_fft2_bf16x6"
        _lib.check(getattr(_lib.lib(), name + "_workspace_bytes")(batch, W, ctypes.byref(n)), name + "_workspace_bytes")
        ws, mark = self._ordered_aux("fft2_tensor_core", int(n.value), stream)
        st = getattr(_lib.lib(), name)(_ptr(x), _ptr(out), batch, W, int(inverse), _ptr(ws), ws.numel(),
                                       stream.cuda_stream)
        mark()
        _lib.check(st, name)
        return out

    @staticmethod
    def _check_inputs(problem, obj, probe, measured, scenarios=1):
        W = problem.window
        want_obj = (problem.obj_ny, problem.obj_nx, problem.n_slices, problem.n_obj_modes)
        if tuple(obj.shape) != want_obj or obj.dtype != torch.complex64 or not obj.is_contiguous():
            raise ValueError("object must be a contiguous complex64 tensor of shape %s" % (want_obj,))
        if scenarios > 1:
            want = (W, W, problem.n_probe_modes, scenarios)
            if tuple(probe.shape) != want or probe.dtype != torch.complex64 or not probe.is_contiguous():
                raise ValueError("probe must be a contiguous complex64 tensor of shape %s" % (want,))
        elif tuple(probe.shape) != (W, W, problem.n_probe_modes) or probe.dtype != torch.complex64 \
                or not probe.is_contiguous():
            raise ValueError("probe must be a contiguous complex64 tensor of shape %s" %
                             ((W, W, problem.n_probe_modes),))
        if measured is not None and (tuple(measured.shape) != (problem.n_positions, W, W) or
                                     measured.dtype != torch.float32 or not measured.is_contiguous()):
            raise ValueError("measured must be a contiguous float32 tensor of shape %s" %
                             ((problem.n_positions, W, W),))
        for t in (obj, probe):
            if not t.is_cuda:
                raise ValueError("inputs must be CUDA tensors")
        if measured is not None and not _readable(measured):
            raise ValueError("measured must be a CUDA tensor or a pinned host tensor (read in place over "
                             "the host link)")


def _readable(t: torch.Tensor) -> bool:
    """Device memory, or pinned host memory that the kernels read in place (the patterns of a
    dataset larger than HBM streamed over the host link, no staging copy)."""
    return t.is_cuda or (t.device.type == "cpu" and t.is_pinned())


_ENGINES = {}


def default_engine(device=None) -> Engine:
    dev = torch.device(device if device is not None else "cuda")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    eng = _ENGINES.get(dev)
    if eng is None:
        eng = _ENGINES[dev] = Engine(dev)
    return eng
