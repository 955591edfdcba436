"""GPU-resident optimizer step around ``loss_and_direction``: L-BFGS with a Wolfe line search.

Restates ``pypty.iterative.bfgs_update`` (``pypty/iterative.py:440-1049``) for the flag set
the GPU path supports, with every array operation on the device:

* ``fourier_clean_`` -- the band limit ``pypty.utils.fourier_clean`` (``utils.py:102-150``)
  of an ``(Ny, Nx, ...)`` complex64 tensor, three HBM passes of strided batched FFTs
  (``pty_fourier_clean``), optionally of ``x + step * dx`` (the trial point) in the same pass;
* ``LBFGS`` -- the state of ``history_bfgs`` (``iterative.py:1055-1103``) kept on the device:
  history pairs (s, y) per variable, rho / alpha / gamma scalars in FP64, the last accepted
  loss and gradients; ``step()`` runs one call of ``bfgs_update``.

The host keeps only the loop control: per line-search trial it reads back the trial loss
and the directional derivative (16 bytes) to take the Wolfe decisions
(``pypty/utils.py:326-368``). The reference's NumPy/CuPy version synchronises on every
scalar reduction.

Variables (segments of the optimizer's vector space, ``pty_vspace_t``): the object
(complex64, inner-product weight 2), the probe (complex64, weight 2) and the sub-pixel
position corrections (float32, weight 1), as ``iterative.py:583-606`` weighs them.
Not supported (``NotImplementedError`` from the callers): phase-only objects, probe
Fourier-phase / amplitude tuning, tilts, static background, aberrations, beam current,
charge flipping, Gaussian filters, object resizing and position puzzling.
"""
from __future__ import annotations

import ctypes
import sys
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .engine import Engine, Geometry, default_engine


def _f32view(t: torch.Tensor) -> torch.Tensor:
    return torch.view_as_real(t).reshape(-1) if t.is_complex() else t.reshape(-1)


def _ptrs(tensors):
    return (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])


def _stream(eng: Engine):
    return torch.cuda.current_stream(eng.device).cuda_stream


def fourier_clean_(x: torch.Tensor, cutoff=None, rolloff=0.0, mask=None, out: torch.Tensor | None = None,
                   dx: torch.Tensor | None = None, step: float = 0.0, engine: Engine | None = None) -> torch.Tensor:
    """out = fourier_clean(x + step * dx) over axes 0, 1 of a complex64 CUDA tensor (any
    trailing axes). ``cutoff``/``rolloff`` follow ``utils.fourier_clean`` in float32
    arithmetic; ``mask``: a (Ny, Nx) mask in fftshifted order instead. out may be x."""
    eng = engine or default_engine(x.device)
    if x.dtype != torch.complex64 or not x.is_cuda or not x.is_contiguous():
        raise TypeError("fourier_clean_ needs a contiguous complex64 CUDA tensor")
    if x.dim() < 2:
        raise ValueError("fourier_clean_ needs at least 2 axes")
    ny, nx = int(x.shape[0]), int(x.shape[1])
    k = int(np.prod(x.shape[2:])) if x.dim() > 2 else 1
    if out is None:
        out = torch.empty_like(x)
    if dx is not None and (dx.shape != x.shape or dx.dtype != x.dtype or not dx.is_contiguous()):
        raise ValueError("dx must match x")
    ws = _clean_tables(eng, ny, nx, cutoff, rolloff, mask)
    _lib.check(_lib.lib().pty_fourier_clean_apply(
        x.data_ptr(), dx.data_ptr() if dx is not None else None, float(step), out.data_ptr(), ny, nx, k,
        ws.data_ptr(), ws.numel(), _stream(eng)), "pty_fourier_clean_apply")
    return out


def _clean_tables(eng: Engine, ny, nx, cutoff, rolloff, mask):
    """Twiddle and band-limit tables of one (ny, nx, cutoff, rolloff), prepared once per
    engine (``pty_fourier_clean_prepare``); a caller-given mask is prepared every call."""
    n = ctypes.c_size_t(0)
    _lib.check(_lib.lib().pty_fourier_clean_workspace_bytes(ny, nx, ctypes.byref(n)),
               "pty_fourier_clean_workspace_bytes (object extents must be powers of two in [64, 8192])")
    if mask is not None:
        m = mask if isinstance(mask, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(
            np.asarray(mask.get() if hasattr(mask, "get") else mask, dtype=np.float32)))
        m = m.to(device=eng.device, dtype=torch.float32).reshape(ny, nx).contiguous()
        ws = eng.aux("fourier_clean_given_mask", int(n.value))
        eng._aux["fourier_clean_mask_src"] = m     # alive until the kernels have read it
        _lib.check(_lib.lib().pty_fourier_clean_prepare(ny, nx, 0.0, 0.0, m.data_ptr(), ws.data_ptr(), ws.numel(),
                                                        _stream(eng)), "pty_fourier_clean_prepare")
        return ws
    c32, r32 = np.float32(cutoff), np.float32(rolloff)
    key = "fourier_clean:%d:%d:%08x:%08x" % (ny, nx, c32.view(np.uint32), r32.view(np.uint32))
    ws = eng._aux.get(key)
    if ws is None:
        ws = eng.aux(key, int(n.value))
        _lib.check(_lib.lib().pty_fourier_clean_prepare(ny, nx, float(c32), float(r32), None, ws.data_ptr(),
                                                        ws.numel(), _stream(eng)), "pty_fourier_clean_prepare")
    return ws


def orthogonalize_modes_(probe: torch.Tensor, engine: Engine | None = None) -> torch.Tensor:
    """Gram-Schmidt over the last axis of a (W, W, Mp) complex64 CUDA probe, in place
    (``pypty/objective.py:1119-1141``). A (W, W, Mp, S) probe of S scenarios is treated as the
    reference treats it: its first S modes, each spanning every pixel of every scenario, are
    orthogonalised (``n_states`` is the last axis, the modes are indexed on the third)."""
    eng = engine or default_engine(probe.device)
    if probe.dim() == 4:
        mp, ns = int(probe.shape[2]), int(probe.shape[3])
        if ns > mp:   # the reference indexes mode ns - 1 of mp modes
            raise IndexError("index %d is out of bounds for axis 2 with size %d" % (mp, mp))
        x = probe.permute(0, 1, 3, 2).contiguous()          # (W, W, S, Mp): modes innermost
        sub = x[..., :ns].contiguous()
        _lib.check(_lib.lib().pty_orthogonalize_modes(sub.data_ptr(), sub.numel() // ns, ns, _stream(eng)),
                   "pty_orthogonalize_modes")
        x[..., :ns] = sub
        probe.copy_(x.permute(0, 1, 3, 2))
        return probe
    mp = int(probe.shape[-1])
    _lib.check(_lib.lib().pty_orthogonalize_modes(probe.data_ptr(), probe.numel() // mp, mp, _stream(eng)),
               "pty_orthogonalize_modes")
    return probe


@dataclass
class LineSearchConfig:
    """Arguments of ``bfgs_update`` that shape the step (``pypty/iterative.py:440``)."""
    update_obj: bool = True
    update_probe: bool = True
    update_pos: bool = False
    # the variants path's extra variables (pypty/iterative.py:477-481): tilt corrections,
    # aberration arrays, beam currents
    update_tilts: bool = False
    update_static_background: bool = False
    update_aberrations: bool = False
    update_beam_current: bool = False
    clean_cutoff: float = np.float32(2 / 3) - np.float32(0.005)   # damping_cutoff - update_extra_cut
    smooth_rolloff: float = 0.0
    lazy_clean: bool = False
    keep_probe_states_orthogonal: bool = False
    aperture: object = None          # clean_grad_ap (probe_reg_weight == inf): cutoff or mask
    wolfe_c1: float = 0.5
    wolfe_c2: float = 0.9
    max_count: int | None = None
    reduce_factor: float = 0.1
    optimism: float = 3
    stepsize_threshold_low: float = 1e-20
    hist_length: int = 10
    verbose: int = 0


@dataclass
class StepResult:
    total_loss: float
    sse: float
    actual_step: float
    count: int
    d_value: float
    new_d_value: float
    accepted: bool
    warnings: list = field(default_factory=list)


class LBFGS:
    """Device-resident L-BFGS / Wolfe line search of ``bfgs_update`` around the fused
    ``loss_and_direction`` (``pty_loss_and_direction``).

    obj (Ny, Nx, Z, Mo) complex64, probe (W, W, Mp) complex64, corr (N, 2) float32 and
    measured (N, W, W) float32 are CUDA tensors; ``problem`` / ``geometry`` describe the
    scan (``engine.make_problem``). ``step()`` updates ``obj``, ``probe`` and ``corr`` in
    place of the attributes (new tensors) and keeps the history on the device.
    """

    HMAX = 64

    # refined variables in the reference's order (iterative.py:597-609): name, inner-product
    # weight (complex segments count twice), state attribute
    SEGMENTS = (("obj", 2.0, "obj"), ("probe", 2.0, "probe"), ("pos", 1.0, "corr"), ("tilts", 1.0, "tcorr"),
                ("static_background", 1.0, "sb"), ("aberrations", 1.0, "ab"), ("beam_current", 1.0, "bc"))

    def __init__(self, problem: _lib.Problem, geometry: Geometry, measured: torch.Tensor, obj: torch.Tensor,
                 probe: torch.Tensor, corr: torch.Tensor, config: LineSearchConfig, engine: Engine | None = None,
                 variant: dict | None = None, tilts: torch.Tensor | None = None,
                 tilts_correction: torch.Tensor | None = None, aberrations: torch.Tensor | None = None,
                 beam_current: torch.Tensor | None = None, static_background: torch.Tensor | None = None):
        self.eng = engine or default_engine(obj.device)
        # keyword arguments of Engine.loss_and_direction_variants (near field, compressed
        # detectors, beam current, aberration plates, tilts), or None for the fused path
        self.variant = variant
        self.problem, self.geo, self.measured = problem, geometry, measured
        self.obj, self.probe, self.corr = obj, probe, corr
        # extra variables of the variants path (device float32): the tilt rows and their
        # refined correction, the static background, the aberration arrays, the beam currents
        self.tilts, self.tcorr, self.ab, self.bc = tilts, tilts_correction, aberrations, beam_current
        self.sb = static_background
        self.cfg = config
        n = ctypes.c_size_t(0)
        _lib.check(_lib.lib().pty_lbfgs_state_bytes(ctypes.byref(n)), "pty_lbfgs_state_bytes")
        self.state = torch.empty(int(n.value), dtype=torch.uint8, device=self.eng.device)
        # pty_lbfgs_read: d_value, new_d_value, gamma[MAX_SEG], dot[MAX_SEG]
        self.read_buf = torch.empty(2 + 2 * _lib.VSPACE_MAX_SEG, dtype=torch.float64, pin_memory=True)
        self._vs_flags = None
        self.reset()

    # ------------------------------------------------------------------ state
    def reset(self):
        """``reset_bfgs_history`` (``pypty/iterative.py:1055-1103``)."""
        self.history = []          # slots, oldest first
        self.pairs = {}            # slot -> (s list, y list)
        self.free = list(range(self.HMAX))
        self.prev = None           # (loss, sse, grad list) of the last accepted point
        self.empty = True
        self._vs_flags = None

    def _flags(self):
        c = self.cfg
        return (c.update_obj, c.update_probe, c.update_pos, c.update_tilts, c.update_static_background,
                c.update_aberrations, c.update_beam_current)

    def _vspace(self):
        flags = self._flags()
        vs = _lib.VSpace()
        names = [nm for (nm, _, _), on in zip(self.SEGMENTS, flags) if on]
        vs.n_seg = len(names)
        vs.obj_seg = names.index("obj") if "obj" in names else -1
        i = 0
        for (nm, w, attr), on in zip(self.SEGMENTS, flags):
            if on:
                vs.n[i] = _f32view(getattr(self, attr)).numel()
                vs.weight[i] = w
                i += 1
        return vs, names, flags

    def _st(self):
        return _stream(self.eng)

    def _clean(self, t, out=None, dx=None, step=0.0):
        return fourier_clean_(t, self.cfg.clean_cutoff, self.cfg.smooth_rolloff, out=out, dx=dx, step=step,
                              engine=self.eng)

    def _clean_aperture(self, t):
        ap = self.cfg.aperture
        if ap is None:
            return t
        if isinstance(ap, (int, float, np.floating)):
            return fourier_clean_(t, ap, 0.0, out=t, engine=self.eng)
        return fourier_clean_(t, mask=ap, out=t, engine=self.eng)

    def _lad(self, x):
        """loss_and_direction at the point x = [obj, probe, corr, tcorr, sb, ab, bc]: returns
        (loss_sse, [object, probe, position, tilt, static-background, aberration, beam-current
        gradients])."""
        p = self.problem
        obj, probe, corr, tcorr, sb, ab, bc = x
        if self.variant is not None:
            c = self.cfg
            kw = dict(self.variant)
            if self.tilts is not None:   # the reference evaluates tilts + tilts_correction (objective.py:343)
                kw["tilts"] = (self.tilts + tcorr) if tcorr is not None else self.tilts   # stays on the device
                kw["step_tilts"] = c.update_tilts
            if ab is not None:
                kw["aberrations"], kw["step_aberrations"] = ab, c.update_aberrations
            if bc is not None:
                kw["beam_current"], kw["step_beam_current"] = bc, c.update_beam_current
            if sb is not None:
                kw["static_background"], kw["step_static_background"] = sb, c.update_static_background
            loss_sse, og, pg, posg, bcg, abg, tg, sbg = self.eng.loss_and_direction_variants(
                p, obj, probe, self.geo, self.measured, pos_correction=corr, **kw)
            return loss_sse, [og, pg, posg, tg, sbg, abg, bcg]
        out = (torch.empty(2, dtype=torch.float64, device=self.eng.device), torch.empty_like(obj),
               torch.empty_like(probe), torch.empty((p.n_positions, 2), dtype=torch.float32, device=self.eng.device))
        loss_sse, og, pg, posg = self.eng.loss_and_direction(p, obj, probe, self.geo, self.measured, out=out,
                                                             pos_correction=corr)
        return loss_sse, [og, pg, posg, None, None, None, None]

    def _point(self):
        return [self.obj, self.probe, self.corr, self.tcorr, self.sb, self.ab, self.bc]

    def _grad_vec(self, grads):
        return [_f32view(gr) for gr, on in zip(grads, self._flags()) if on]

    def _read(self):
        _lib.check(_lib.lib().pty_lbfgs_read(self.state.data_ptr(),
                                             ctypes.cast(self.read_buf.data_ptr(), ctypes.POINTER(ctypes.c_double)),
                                             self._st()), "pty_lbfgs_read")
        return self.read_buf.numpy().copy()

    def _post_grad(self, og, pg):
        """Band limits of a fresh gradient (iterative.py:528-548, 776-797)."""
        c = self.cfg
        if c.aperture is not None:
            self._clean_aperture(pg)
        if c.update_probe:
            self._clean(pg, out=pg)
        if not c.lazy_clean and c.update_obj:
            self._clean(og, out=og)

    # ------------------------------------------------------------------ one call of bfgs_update
    def step(self, actual_step=1) -> StepResult:
        c = self.cfg
        lib = _lib.lib()
        st = self._st()
        warnings = []
        vs, names, flags = self._vspace()
        if self._vs_flags is not None and self._vs_flags != flags:
            self.reset()         # the set of refined variables changed: the history no longer applies
        if self.empty:
            _lib.check(lib.pty_lbfgs_reset(ctypes.byref(vs), self.state.data_ptr(), st), "pty_lbfgs_reset")
        self._vs_flags = flags
        # pre-clean of the current point (iterative.py:485-514)
        if c.aperture is not None:
            self._clean_aperture(self.probe)
        if c.update_probe:
            if self.probe.shape[-1] > 1 and c.keep_probe_states_orthogonal:
                orthogonalize_modes_(self.probe, self.eng)
            self._clean(self.probe, out=self.probe)
        if c.update_obj and not c.lazy_clean:
            self._clean(self.obj, out=self.obj)
        flags = self._flags()
        point = self._point()
        qs = [torch.empty_like(t) if on else None for t, on in zip(point, flags)]
        q_obj = qs[0]
        qv = [_f32view(t) for t in qs if t is not None]
        if self.empty:
            loss_sse, grads = self._lad(point)
            self._post_grad(grads[0], grads[1])
            g = self._grad_vec(grads)
            _lib.check(lib.pty_lbfgs_first_direction(ctypes.byref(vs), _ptrs(g), _ptrs(qv), self.state.data_ptr(),
                                                     st), "pty_lbfgs_first_direction")
            ls = loss_sse.cpu().numpy()
            total_loss, sse = float(ls[0]), float(ls[1])
            self.empty = False
        else:
            total_loss, sse, grads = self.prev
            pg = grads[1]
            if c.aperture is not None:
                self._clean_aperture(pg)
            if c.update_probe:
                self._clean(pg, out=pg)
            g = self._grad_vec(grads)
            m = len(self.history)
            svec = [p for sl in self.history for p in self.pairs[sl][0]]
            yvec = [p for sl in self.history for p in self.pairs[sl][1]]
            slots = (ctypes.c_int32 * m)(*self.history)
            _lib.check(lib.pty_lbfgs_two_loop(ctypes.byref(vs), _ptrs(g), _ptrs(qv), m, _ptrs(svec), _ptrs(yvec),
                                              slots, self.state.data_ptr(), st), "pty_lbfgs_two_loop")
            if c.update_obj and not c.lazy_clean:
                self._clean(q_obj, out=q_obj)
            _lib.check(lib.pty_lbfgs_dot(ctypes.byref(vs), _ptrs(qv), _ptrs(g), 0, self.state.data_ptr(), st),
                       "pty_lbfgs_dot")
        if total_loss != total_loss:
            raise ValueError('A very specific bad thing. Loss is Nan.')
        d_value = float(self._read()[0])
        if d_value >= 0:     # iterative.py:691-700
            sys.stdout.write("\n\n\nWarning! Positive dir-derivative, using normal gradient-descent!\n\n\n\n\n\n")
            sys.stdout.flush()
            warnings.append("\n\\Positive dir-derivative, using normal gradient-descent!")
            _lib.check(lib.pty_lbfgs_steepest(ctypes.byref(vs), _ptrs(g), _ptrs(qv), self.state.data_ptr(), st),
                       "pty_lbfgs_steepest")
            d_value = float(self._read()[0])
        # ------------------------------------------------------------ line search (iterative.py:733-837)
        count = -1
        new = [torch.empty_like(t) if on else t for t, on in zip(point, flags)]
        while True:
            count += 1
            for i, on in enumerate(flags):
                if not on:
                    continue
                if i == 0 and not c.lazy_clean:   # the object trial point is band-limited (iterative.py:759-766)
                    self._clean(self.obj, out=new[0], dx=q_obj, step=float(np.float32(actual_step)))
                else:
                    self._axpy1(new[i], point[i], qs[i], actual_step)
            loss_sse, ngrads = self._lad(new)
            self._post_grad(ngrads[0], ngrads[1])
            ng = self._grad_vec(ngrads)
            _lib.check(lib.pty_lbfgs_dot(ctypes.byref(vs), _ptrs(qv), _ptrs(ng), 1, self.state.data_ptr(), st),
                       "pty_lbfgs_dot")
            new_d_value = float(self._read()[1])
            ls = loss_sse.cpu().numpy()
            new_total_loss, new_sse = float(ls[0]), float(ls[1])
            if new_total_loss != new_total_loss:
                raise ValueError('A very specific bad thing. Loss is Nan.')
            wolfe_1 = new_total_loss <= total_loss + c.wolfe_c1 * actual_step * d_value
            wolfe_2 = -1 * new_d_value <= -1 * d_value * c.wolfe_c2
            if c.verbose >= 3:
                sys.stdout.write("\nLinesearch iteration %d. This loss is %.3e. Loss change is %.3e. Dir-derivative "
                                 "is %.3e. New dir-derivative is %.3e, This step is %.3e." % (
                                     count, total_loss, total_loss - new_total_loss, d_value, new_d_value,
                                     actual_step))
            if wolfe_1 and wolfe_2:
                break
            if not wolfe_1 and wolfe_2:
                actual_step *= c.reduce_factor
            if not wolfe_2 and wolfe_1:
                actual_step *= c.optimism
            if not (wolfe_2 or wolfe_1):
                actual_step = type(actual_step)(10 ** (np.random.uniform(0, 20) - 20))
            if c.max_count is not None and count > c.max_count:
                break
            if actual_step < c.stepsize_threshold_low:
                break
        if not wolfe_1:       # iterative.py:838-844
            sys.stdout.write('\nWARNING! The sufficient loss descrese is not achieved, the update is regected, '
                             'keeping the the same step! Resetting the history! Please terminate if this message '
                             'appears during the next epoch!\n')
            sys.stdout.flush()
            warnings.append("\nSufficient loss descrese is not achieved, the update is regected")
            self.reset()
            return StepResult(total_loss, sse, actual_step, count, d_value, new_d_value, False, warnings)
        # ------------------------------------------------------------ history (iterative.py:849-931)
        slot = self.free.pop(0)
        s_t = [torch.empty_like(t) for t in qv]
        y_t = [torch.empty_like(t) for t in qv]
        _lib.check(lib.pty_lbfgs_accept(ctypes.byref(vs), float(actual_step), _ptrs(qv), _ptrs(g), _ptrs(ng),
                                        _ptrs(s_t), _ptrs(y_t), slot, self.state.data_ptr(), st), "pty_lbfgs_accept")
        self.pairs[slot] = (s_t, y_t)
        self.history.append(slot)
        self.prev = (new_total_loss, new_sse, ngrads)
        while len(self.history) > c.hist_length:
            old = self.history.pop(0)
            del self.pairs[old]
            self.free.append(old)
        for (_, _, attr), on, t in zip(self.SEGMENTS, flags, new):
            if on:
                setattr(self, attr, t)
        return StepResult(total_loss, sse, actual_step, count, d_value, new_d_value, True, warnings)

    def _axpy1(self, out, a, b, step):
        vs = _lib.VSpace()
        vs.n_seg = 1
        vs.obj_seg = -1
        av = _f32view(a)
        vs.n[0] = av.numel()
        vs.weight[0] = 1.0
        _lib.check(_lib.lib().pty_lbfgs_axpy(ctypes.byref(vs), _ptrs([_f32view(out)]), _ptrs([av]),
                                             _ptrs([_f32view(b)]), float(np.float32(step)), self._st()),
                   "pty_lbfgs_axpy")

    def gammas(self):
        """Current Barzilai-Borwein gamma per refined variable (host read, synchronising)."""
        r = self._read()
        names = self._vspace()[1]
        return {nm: float(r[2 + i]) for i, nm in enumerate(names)}
