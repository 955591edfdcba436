"""Drop-in ``loss_and_direction`` with the reference's signature, on the GPU path.

``loss_and_direction`` takes exactly the arguments of ``pypty.objective.loss_and_direction``
(``pypty/objective.py:47``), in the same order, and returns the same 10-tuple
(``pypty/objective.py:967``). Installing it in place of the reference function
(``pypty_gb300.shim.install``) lets ``pypty.iterative.run`` drive the GB300 kernels.

Supported flag set: ``propmethod="multislice"``, one slice distance or one per slice step
(``this_distances`` with more than one entry, ``multislice_core.py:69-74``), algorithms ``lsq_sqrt``,
``ml``, ``lsq``, ``lsq_sqrt_2`` on the fused path; with any of far-field or near-field
propagation (one defocus or one per position, ``Cs``; ``pypty/objective.py:413-418, 504-508``), the compressed-detector
algorithms with ``masks`` (``objective.py:560-585``), beam-current fluctuations and their
gradient, aberration arrays with markers and their gradient, or beam tilts (``tilt_mode``
0-4, one tilt row or one per position, with the tilt gradient) on the variants path
(``pty_loss_and_direction_variants``), which also takes the detector upsampling
(``upsample_pattern``, ``objective.py:523-524, 590-591``) and a 2D static background with
its gradient (``objective.py:359-361, 525-526, 588-589``), and several probe scenarios (a 4D
probe with ``probe_marker``, ``objective.py:355-356, 443-444, 700-701``). No phase plates,
data binning (the reference raises on it), near-field ``alpha_near_field`` (the reference
raises on it) or regularisers. The per-batch measured-data preprocessing
(``data_pad`` with or without ``use_padded_intensity``, ``data_shift_vector``,
``data_multiplier``) runs on the fly on the variants path; with ``load_one_by_one`` the
patterns stay in pinned host memory and the kernels read them in place. Any other combination raises
``NotImplementedError`` naming the flag: the product path never falls back to a CPU
implementation.
"""
from __future__ import annotations

import warnings

import numpy as np
import torch

from . import _lib
from .engine import Geometry, default_engine, make_problem

N_CONSTRAINTS = 14   # entries of constraint_contributions (pypty/objective.py:768-921)


class ComputePrecisionWarning(RuntimeWarning):
    """Inputs or ``default_complex`` ask for complex128, but the GPU path computes in
    complex64 (the results come back in the caller's dtype)."""


def _precision_check(this_obj, full_probe, default_complex):
    """The reference's default dtype is "double" (``pypty/iterative.py:58-60``: complex128
    arrays, ``default_complex`` complex128). The kernels compute in complex64 with FP64 loss
    and step-size reductions; this warns (once per call site, Python's default filter) when
    double precision was asked for, instead of narrowing silently."""
    def is_c128(x):
        try:
            return np.dtype(x) == np.complex128
        except TypeError:
            return False
    asked = is_c128(default_complex) or any(
        is_c128(getattr(a, "dtype", None)) or (isinstance(a, torch.Tensor) and a.dtype == torch.complex128)
        for a in (this_obj, full_probe))
    if asked:
        warnings.warn("pypty_gb300 computes the loss and gradients in complex64 (FP64 loss and "
                      "step-size reductions); complex128 inputs are rounded to complex64 and the "
                      "results returned as complex128", ComputePrecisionWarning, stacklevel=3)
    return asked


def _unsupported(cond, what):
    if cond:
        raise NotImplementedError("pypty_gb300 GPU path does not implement %s" % what)


def _is_zero(x):
    if x is None:
        return True
    try:
        return float(np.sum(np.abs(np.asarray(x)))) == 0.0
    except (TypeError, ValueError):
        return False


def _to_numpy(a):
    if isinstance(a, torch.Tensor):
        return a.detach().cpu().numpy()
    if hasattr(a, "get"):          # a CuPy array
        return a.get()
    return np.asarray(a)


def _device_tensor(a, dtype, device):
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(_to_numpy(a))).to(device=device, dtype=dtype)


_PINNED = {}


def measured_tensor(measured_array, device, load_one_by_one):
    """The measured patterns as the kernels read them. With ``load_one_by_one`` (the
    reference keeps the dataset in host memory and copies each batch, ``objective.py:398-409``)
    a host array is copied into a pinned buffer and read in place by the kernels over the host
    link, so a dataset larger than HBM needs no device copy; otherwise it is copied to the
    device. The reference reads the caller's array on every call, so the pinned buffer is
    refreshed from it on every call too (a host copy), unless the array is read-only and
    cannot have changed since the buffer was filled."""
    if isinstance(measured_array, torch.Tensor) and (measured_array.is_cuda or measured_array.is_pinned()):
        return measured_array.to(torch.float32).contiguous()
    if not load_one_by_one:
        return _device_tensor(measured_array, torch.float32, device)
    key = id(measured_array)
    hit = _PINNED.get(key)
    host = _to_numpy(measured_array)
    if hit is None or hit[0] is not measured_array or tuple(hit[1].shape) != tuple(host.shape):
        _PINNED.clear()                      # one dataset pinned at a time
        pinned = torch.empty(tuple(host.shape), dtype=torch.float32, pin_memory=True)
        np.copyto(pinned.numpy(), host, casting="unsafe")
        _PINNED[key] = hit = (measured_array, pinned)
    elif not (isinstance(host, np.ndarray) and not host.flags.writeable):
        np.copyto(hit[1].numpy(), host, casting="unsafe")   # the caller may have changed it in place
    return hit[1]


def prepare(this_obj, full_probe, this_pos_array, this_pos_correction, this_tilt_array,
                       this_tilts_correction, this_distances, edge_slice_thickness_multiplier,
                       measured_array, algorithm_type, this_wavelength, this_step_probe, this_step_obj,
                       this_step_pos_correction, this_step_tilts, masks, pixel_size_x_A, pixel_size_y_A,
                       recon_type, Cs, defocus_array, alpha_near_field, damping_cutoff_multislice,
                       smooth_rolloff, propmethod, this_chopped_sequence, load_one_by_one, data_multiplier,
                       data_pad, phase_plate_in_h5, this_loss_weight, data_bin, data_shift_vector,
                       upsample_pattern, static_background, this_step_static_background, tilt_mode,
                       aberration_marker, probe_marker, aberrations_array, compute_batch, phase_only_obj,
                       beam_current, this_beam_current_step, this_step_aberrations_array, default_float,
                       default_complex, xp, is_first_epoch, scan_size, scan_step_A,
                       fast_axis_reg_weight_positions, slow_axis_reg_weight_positions,
                       slow_axis_reg_weight_tilts, current_deformation_reg_weight_positions,
                       current_deformation_reg_weight_tilts, fast_axis_reg_weight_tilts, aperture_mask,
                       probe_reg_weight, current_window_weight, current_window, phase_norm_weight,
                       abs_norm_weight, atv_weight, atv_q, atv_p, mixed_variance_weight, mixed_variance_sigma,
                       wedge_mu, beta_wedge, probe_mod_reg_weight, probe_mod_tol, smart_memory, print_flag,
                       data_simulation_flag, data_simulation_exitwave, use_padded_intensity):
    """Check the arguments of ``loss_and_direction`` against the supported flag set and
    build the C-ABI problem and scan geometry: returns (problem, geometry, variant) where
    variant is None for the fused far-field path, else the keyword arguments of
    ``Engine.loss_and_direction_variants``. ``NotImplementedError`` names the first
    unsupported flag. Warns ``ComputePrecisionWarning`` when complex128 is asked for."""
    _precision_check(this_obj, full_probe, default_complex)
    _unsupported(recon_type not in _lib.RECON_TYPES, "recon_type=%r" % (recon_type,))
    _unsupported(propmethod != "multislice", "propmethod=%r" % (propmethod,))
    compressed = algorithm_type in _lib.COMPRESSED_ALGORITHMS
    _unsupported(algorithm_type not in _lib.ALGORITHMS and not compressed, "algorithm_type=%r" % (algorithm_type,))
    _unsupported(compressed and masks is None, "compressed algorithms without masks")
    tmode = 0 if tilt_mode is None else int(tilt_mode)
    _unsupported(tmode not in (0, 1, 2, 3, 4), "tilt_mode=%r" % (tilt_mode,))
    # the reference adds the correction in the default float type (objective.py:343, 348)
    tilts = np.asarray(_to_numpy(this_tilt_array), dtype=np.float32) + \
        np.asarray(_to_numpy(this_tilts_correction), dtype=np.float32)
    n_pos = int(np.asarray(_to_numpy(this_pos_array)).shape[0])
    _unsupported(tilts.ndim != 2 or tilts.shape[1] != 6 or tilts.shape[0] not in (1, n_pos),
                 "tilt arrays that are not one row or one row per position")
    tilted = tmode != 0 or bool(this_step_tilts) or not _is_zero(tilts)
    dists = np.asarray(_to_numpy(this_distances), dtype=np.float32).reshape(-1)
    n_slices = int(tuple(this_obj.shape)[2]) if len(tuple(this_obj.shape)) == 4 else 1
    # more than one entry: step z uses entry z (multislice_core.py:69-74); the reference indexes
    # past a shorter array
    _unsupported(dists.shape[0] > 1 and dists.shape[0] < n_slices - 1,
                 "this_distances with fewer than n_slices - 1 entries (the reference raises IndexError)")
    _unsupported(phase_plate_in_h5 is not None, "phase plates")
    # a 4D probe with probe_marker: one probe per scenario (multiple_scenarios, objective.py:285)
    scen = probe_marker is not None and len(tuple(full_probe.shape)) == 4
    near = recon_type == "near_field"
    dfa = np.asarray(_to_numpy(defocus_array), dtype=np.float32).reshape(-1)
    if near:
        # one defocus per position (objective.py:413-418): indexed by position
        _unsupported(dfa.shape[0] != 1 and dfa.shape[0] != n_pos,
                     "defocus_array that is neither one value nor one per position")
        _unsupported(float(alpha_near_field) > 0, "alpha_near_field > 0 (the reference raises on it)")
    _unsupported(aberrations_array is not None and aberration_marker is None, "aberrations without markers")
    _unsupported(bool(this_step_aberrations_array) and aberrations_array is None, "aberration steps without arrays")
    _unsupported(bool(this_beam_current_step) and beam_current is None, "beam-current steps without currents")
    # a scalar static background cannot be indexed by the reference (objective.py:361); zero
    # is read here as no background
    has_bg = static_background is not None and not (np.ndim(_to_numpy(static_background)) == 0
                                                    and _is_zero(static_background))
    _unsupported(has_bg and np.ndim(_to_numpy(static_background)) != 2, "a static background that is not 2D")
    _unsupported(bool(this_step_static_background) and not has_bg, "static-background steps without a background")
    # the reference's binning loop indexes an undefined name (utils.py:643: i2), so it raises
    _unsupported(int(data_bin) != 1, "data binning (the reference raises NameError on it)")
    up = max(int(upsample_pattern), 1)
    padded = True if use_padded_intensity is None else bool(use_padded_intensity)
    _unsupported(compressed and up != 1, "upsample_pattern with compressed detectors")
    _unsupported(has_bg and (up != 1 or (int(data_pad) != 0 and not padded)),
                 "a static background with upsampling or a cropped pattern (the reference's shapes do not broadcast)")
    _unsupported(compressed and int(data_pad) != 0, "data_pad with compressed detectors")
    prep = not compressed and (int(data_pad) != 0 or not _is_zero(data_shift_vector) or float(data_multiplier) != 1.0)
    # data_simulation_flag: the model patterns (fused path) or the exit waves
    # (data_simulation_exitwave, variants path) are also saved to that file
    # (objective.py:286-293, 518-522, 744-749)
    exitwave = bool(data_simulation_flag) and bool(data_simulation_exitwave)
    for name, w in [("fast_axis_reg_weight_positions", fast_axis_reg_weight_positions),
                    ("slow_axis_reg_weight_positions", slow_axis_reg_weight_positions),
                    ("current_deformation_reg_weight_positions", current_deformation_reg_weight_positions)]:
        _unsupported(bool(this_step_pos_correction) and w != 0, name)
    for name, w in [("phase_norm_weight", phase_norm_weight), ("abs_norm_weight", abs_norm_weight),
                    ("atv_weight", atv_weight), ("wedge_mu", wedge_mu)]:
        _unsupported(w != 0, name)
    for name, w in [("probe_reg_weight", probe_reg_weight), ("current_window_weight", current_window_weight),
                    ("probe_mod_reg_weight", probe_mod_reg_weight)]:
        _unsupported(bool(this_step_probe) and w != 0, name)
    obj_shape = tuple(this_obj.shape)
    _unsupported(len(obj_shape) != 4, "objects that are not 4D (y, x, slice, mode)")
    _unsupported(len(tuple(full_probe.shape)) != (4 if scen else 3),
                 "probes that are not 3D (y, x, mode), or 4D (y, x, mode, scenario) with probe_marker")
    _unsupported(mixed_variance_weight != 0 and obj_shape[3] > 1, "mixed_variance_weight")
    W = int(full_probe.shape[0])
    Mp = int(full_probe.shape[2])
    geo = Geometry.make(_to_numpy(this_pos_array), _to_numpy(this_pos_correction),
                        _to_numpy(this_chopped_sequence))
    problem = make_problem(
        W, obj_shape, Mp, geo, algorithm=algorithm_type, wavelength=float(this_wavelength),
        pixel_size_x=float(pixel_size_x_A), pixel_size_y=float(pixel_size_y_A),
        slice_distance=float(dists[0]), slice_distances=dists if dists.shape[0] > 1 else None,
        edge_mult=float(edge_slice_thickness_multiplier),
        damping_cutoff=None if damping_cutoff_multislice is None else float(damping_cutoff_multislice),
        smooth_rolloff=float(smooth_rolloff), loss_weight=float(this_loss_weight),
        compute_batch=int(compute_batch), step_obj=bool(this_step_obj), step_probe=bool(this_step_probe),
        step_pos=bool(this_step_pos_correction))
    variant = None
    if near or compressed or prep or beam_current is not None or aberrations_array is not None or tilted \
            or up != 1 or has_bg or scen or exitwave:
        variant = dict(recon_type=recon_type,
                       defocus=float(dfa[0]) if near else 0.0,
                       defocus_per_position=dfa if near and dfa.shape[0] > 1 else None,
                       cs=float(Cs) if near else 0.0, tilts=tilts, tilt_mode=tmode,
                       step_tilts=bool(this_step_tilts),
                       masks=None if not compressed else _to_numpy(masks),
                       beam_current=None if beam_current is None else _to_numpy(beam_current),
                       step_beam_current=bool(this_beam_current_step),
                       aberrations=None if aberrations_array is None else _to_numpy(aberrations_array),
                       aberration_marker=None if aberration_marker is None else _to_numpy(aberration_marker),
                       step_aberrations=bool(this_step_aberrations_array),
                       data_pad=0 if compressed else int(data_pad),
                       use_padded_intensity=padded,
                       data_shift_vector=(0, 0) if compressed else tuple(int(x) for x in data_shift_vector),
                       data_multiplier=1.0 if compressed else float(data_multiplier),
                       upsample_pattern=up,
                       static_background=_to_numpy(static_background) if has_bg else None,
                       step_static_background=bool(this_step_static_background) and has_bg,
                       probe_marker=_to_numpy(probe_marker) if scen else None)
    return problem, geo, variant


def loss_and_direction(this_obj, full_probe, this_pos_array, this_pos_correction, this_tilt_array,
                       this_tilts_correction, this_distances, edge_slice_thickness_multiplier,
                       measured_array, algorithm_type, this_wavelength, this_step_probe, this_step_obj,
                       this_step_pos_correction, this_step_tilts, masks, pixel_size_x_A, pixel_size_y_A,
                       recon_type, Cs, defocus_array, alpha_near_field, damping_cutoff_multislice,
                       smooth_rolloff, propmethod, this_chopped_sequence, load_one_by_one, data_multiplier,
                       data_pad, phase_plate_in_h5, this_loss_weight, data_bin, data_shift_vector,
                       upsample_pattern, static_background, this_step_static_background, tilt_mode,
                       aberration_marker, probe_marker, aberrations_array, compute_batch, phase_only_obj,
                       beam_current, this_beam_current_step, this_step_aberrations_array, default_float,
                       default_complex, xp, is_first_epoch, scan_size, scan_step_A,
                       fast_axis_reg_weight_positions, slow_axis_reg_weight_positions,
                       slow_axis_reg_weight_tilts, current_deformation_reg_weight_positions,
                       current_deformation_reg_weight_tilts, fast_axis_reg_weight_tilts, aperture_mask,
                       probe_reg_weight, current_window_weight, current_window, phase_norm_weight,
                       abs_norm_weight, atv_weight, atv_q, atv_p, mixed_variance_weight, mixed_variance_sigma,
                       wedge_mu, beta_wedge, probe_mod_reg_weight, probe_mod_tol, smart_memory, print_flag,
                       data_simulation_flag, data_simulation_exitwave, use_padded_intensity):
    """GPU restatement of ``pypty/objective.py:47-967`` (see the module docstring for the
    supported flag set). Returns (loss, sse, object_grad, probe_grad, pos_grad, tilts_grad,
    static_background_grad, aberrations_array_grad, beam_current_grad,
    constraint_contributions) with the reference's shapes. Arrays come back as NumPy arrays
    when the object was given as a NumPy array, else as CUDA tensors.
    """
    args = dict(locals())
    problem, geo, variant = prepare(**args)
    obj_is_numpy = not isinstance(this_obj, torch.Tensor)
    in_dtype = this_obj.dtype
    eng = default_engine()
    dev = eng.device
    obj_d = _device_tensor(this_obj, torch.complex64, dev)
    probe_d = _device_tensor(full_probe, torch.complex64, dev)
    meas_d = measured_tensor(measured_array, dev, bool(load_one_by_one))
    bc_grad, ab_grad, sb_grad = 0, 0, 0
    tilts_grad = np.zeros_like(_to_numpy(this_tilts_correction))    # objective.py:380
    if problem.n_sequence == 0:
        # no positions: the batch loop does not run and every accumulator stays zero
        # (objective.py:372-382); the variant accumulators are zeros shaped like their inputs
        variant = None
        if beam_current is not None:
            bc_grad = np.zeros_like(_to_numpy(beam_current))
        if aberrations_array is not None:
            ab_grad = np.zeros_like(_to_numpy(aberrations_array))
        if static_background is not None and np.ndim(_to_numpy(static_background)) == 2:
            sb_grad = np.zeros_like(_to_numpy(static_background))
        problem.algorithm = min(int(problem.algorithm), 3)   # the loss is not evaluated
        W = problem.window   # no pattern is read: any measured array of the checked shape
        meas_d = torch.empty((problem.n_positions, W, W), dtype=torch.float32, device=dev)
    sim_exit = None
    if data_simulation_flag and data_simulation_exitwave and variant is not None:
        sim_exit = torch.empty((problem.n_sequence, problem.n_probe_modes, problem.n_obj_modes, problem.window,
                                problem.window), dtype=torch.complex64, device=dev)
        variant = dict(variant, exit_waves=sim_exit)
    if variant is None:
        loss_sse, og, pg, posg = eng.loss_and_direction(problem, obj_d, probe_d, geo, meas_d)
    else:
        kw = dict(variant)
        for k, dt in (("masks", torch.float32), ("beam_current", torch.float32), ("aberrations", torch.float32),
                      ("aberration_marker", torch.int32), ("static_background", torch.float32),
                      ("defocus_per_position", torch.float32), ("probe_marker", torch.int32)):
            if kw[k] is not None:
                kw[k] = _device_tensor(kw[k], dt, dev)
        loss_sse, og, pg, posg, bcg, abg, tg, sbg = eng.loss_and_direction_variants(problem, obj_d, probe_d, geo,
                                                                                    meas_d, **kw)
        # objective.py:377: zeros shaped like the background, 0 without one
        if kw["static_background"] is not None:
            sb_grad = np.zeros_like(_to_numpy(static_background)) if sbg is None else \
                sbg.cpu().numpy().astype(_to_numpy(static_background).dtype, copy=False)
        if tg is not None:
            tilts_grad = tg.cpu().numpy().astype(_to_numpy(this_tilts_correction).dtype, copy=False)
        # zero-initialised accumulators of the reference (objective.py:381-382)
        if beam_current is not None:
            bc_grad = np.zeros_like(_to_numpy(beam_current)) if bcg is None else \
                bcg.cpu().numpy().astype(_to_numpy(beam_current).dtype, copy=False)
        if aberrations_array is not None:
            ab_grad = np.zeros_like(_to_numpy(aberrations_array)) if abg is None else \
                abg.cpu().numpy().astype(_to_numpy(aberrations_array).dtype, copy=False)
    if sim_exit is not None:
        # sim_patterns[tcs] = this_exit_wave, complex128 (N, W, W, Mp, Mo), then np.save
        # (objective.py:289-291, 518-520, 744-749)
        ew = sim_exit.permute(0, 3, 4, 1, 2).cpu().numpy().astype(np.complex128)
        seq = np.asarray(_to_numpy(this_chopped_sequence))
        sim = np.zeros((seq.shape[0],) + ew.shape[1:], dtype=np.complex128)
        sim[seq] = ew
        np.save(data_simulation_flag, sim)
    elif data_simulation_flag:
        _unsupported(variant is not None, "data_simulation_flag with the variants path's flags")
        # sim_patterns[tcs] = this_pattern over every batch, then np.save (objective.py:518-522,
        # 744-749): float64, indexed by the sequence's position entries
        pat = eng.simulate(problem, obj_d, probe_d, geo).cpu().numpy()
        seq = np.asarray(_to_numpy(this_chopped_sequence))
        sim = np.zeros((seq.shape[0],) + pat.shape[1:], dtype=np.float64)
        sim[seq] = pat
        np.save(data_simulation_flag, sim)
    ls = loss_sse.cpu().numpy()
    loss, sse = float(ls[0]), float(ls[1])
    if loss != loss:
        raise ValueError('A very specific bad thing. Loss is Nan.')   # objective.py:925-926
    if not this_step_probe:
        pg = torch.zeros((1,) + tuple(pg.shape), dtype=pg.dtype, device=pg.device)  # objective.py:747-751
    constraints = np.zeros(N_CONSTRAINTS)
    if obj_is_numpy:
        og_out = og.cpu().numpy().astype(in_dtype, copy=False)
        pg_out = pg.cpu().numpy().astype(np.asarray(full_probe).dtype, copy=False)
        posg_out = posg.cpu().numpy().astype(np.asarray(_to_numpy(this_pos_correction)).dtype, copy=False)
    else:
        og_out, pg_out, posg_out = og, pg, posg
    return loss, sse, og_out, pg_out, posg_out, tilts_grad, sb_grad, ab_grad, bc_grad, constraints
