"""``bfgs_update`` and ``reset_bfgs_history`` with the reference's signatures.

``bfgs_update`` takes exactly the arguments of ``pypty.iterative.bfgs_update``
(``pypty/iterative.py:440``) and, like it, reads and writes module-level variables
(``obj``, ``probe``, ``positions``, ``positions_correction``, ``tilts``,
``tilts_correction``, ``static_background``, ``aberrations_array``, ``beam_current``,
``history_bfgs``). ``bind(module)`` returns the same function working on another module's
variables: ``pypty_gb300.shim.install(pypty, iterative=True)`` binds it to
``pypty.iterative`` so that the reference's ``run`` loop drives it.

The update runs on the device (``pypty_gb300.optim.LBFGS``): the history pairs, gradients
and every scalar of the recursion stay in GPU memory between calls; the arrays in the
module variables are read at the start of each call and written back at its end, in the
container type they came in (NumPy arrays or CUDA tensors). The loss and gradients come
from the fused ``pty_loss_and_direction`` with the arguments the reference passes
(``pypty/iterative.py:524,773``; ``smooth_rolloff`` 0 for the loss).

Supported: object, probe and position-correction refinement and, on the variants path, tilt
correction, static-background, aberration-array and beam-current refinement; ``lazy_clean``,
``keep_probe_states_orthogonal``, ``probe_reg_weight = inf`` (aperture-cleaned probe
gradients), ``smart_memory`` (same arithmetic), ``hist_length``, Wolfe constants,
``max_count``, ``reduce_factor``, ``optimism``, ``stepsize_threshold_low``, and every
``loss_and_direction`` flag of ``pypty_gb300.objective``. Other options raise
``NotImplementedError`` naming the option.
"""
from __future__ import annotations

import functools
import inspect
import sys

import numpy as np
import torch

from . import objective
from .engine import default_engine
from .optim import LBFGS, LineSearchConfig

# module variables of the reference (pypty/iterative.py:18-30)
obj = None
probe = None
positions = None
positions_correction = None
tilts = None
tilts_correction = None
static_background = None
aberrations_array = None
beam_current = None
history_bfgs = None

_STATES = {}


def _unsupported(cond, what):
    if cond:
        raise NotImplementedError("pypty_gb300 bfgs_update does not implement %s" % what)


def _fresh_history():
    """The dictionary ``reset_bfgs_history`` builds (``pypty/iterative.py:1065-1098``);
    the pairs themselves live on the device."""
    h = {k: [] for k in ["obj_hist_s", "probe_hist_s", "positions_hist_s", "tilts_hist_s", "beam_current_hist_s",
                         "aberrations_hist_s", "static_background_hist_s", "obj_hist_y", "probe_hist_y",
                         "positions_hist_y", "tilts_hist_y", "beam_current_hist_y", "aberrations_hist_y",
                         "static_background_hist_y", "rho_hist"]}
    h.update({"prev_loss": None, "prev_sse": None, "obj_grad": None, "probe_grad": None, "pos_grad": None,
              "tilt_grad": None, "beam_current_grad": None, "aberrations_grad": None,
              "static_background_grad": None, "empty_hist": True, "gamma_obj": 1, "gamma_probe": 1,
              "gamma_pos": 1, "gamma_tilts": 1, "gamma_static": 1, "gamma_aberrations": 1,
              "gamma_beam_current": 1})
    return h


def reset_bfgs_history():
    """``pypty/iterative.py:1055-1103``: forget the L-BFGS history of this module."""
    global history_bfgs
    history_bfgs = _fresh_history()
    st = _STATES.get(id(sys.modules[__name__]))
    if st is not None and st.get("opt") is not None:
        st["opt"].reset()


def _to_device(a, dtype, dev):
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=dtype).contiguous().clone()
    host = a.get() if hasattr(a, "get") else np.asarray(a)
    return torch.from_numpy(np.ascontiguousarray(host)).to(device=dev, dtype=dtype)


def _like(t, ref):
    """Return device tensor t in the container and dtype of ref."""
    if isinstance(ref, torch.Tensor):
        return t.to(ref.dtype)
    host = ref.get() if hasattr(ref, "get") else np.asarray(ref)
    return t.cpu().numpy().astype(host.dtype, copy=False)


def _impl(ns, a):
    update_obj = a["this_step_obj"] > 0
    update_probe = a["this_step_probe"] > 0
    update_pos = a["this_step_pos_correction"] > 0
    update_tilts = a["this_step_tilts"] > 0
    update_ab = a["this_step_aberrations_array"] > 0
    update_bc = a["this_beam_current_step"] > 0
    update_sb = a["this_step_static_background"] > 0
    _unsupported(update_sb and getattr(ns, "static_background", None) is None,
                 "static-background refinement without a background")
    _unsupported(update_ab and getattr(ns, "aberrations_array", None) is None, "aberration refinement without arrays")
    _unsupported(update_bc and getattr(ns, "beam_current", None) is None, "beam-current refinement without currents")
    _unsupported(bool(a["phase_only_obj"]), "phase_only_obj")
    _unsupported(bool(a["data_simulation_flag"]), "data_simulation_flag inside bfgs_update")
    _unsupported(bool(a["tune_only_probe_phase"]) or bool(a["tune_only_probe_abs"]),
                 "tune_only_probe_phase / tune_only_probe_abs")
    _unsupported(update_obj and bool(a["do_charge_flip"]), "do_charge_flip")
    _unsupported(update_obj and bool(a["current_gaussian_filter"] or a["current_apply_gaussian_filter_amplitude"]),
                 "Gaussian object filters")
    _unsupported(update_pos and bool(a["dynamically_resize_yx_object"]), "dynamically_resize_yx_object")
    _unsupported(update_pos and bool(a["pos_puzzling"]), "pos_puzzling")
    _unsupported(len(tuple(ns.probe.shape)) == 4 and a["probe_marker"] is None,
                 "a 4D probe without probe_marker")
    probe_reg_weight = a["probe_reg_weight"]
    aperture = None
    if probe_reg_weight == np.inf:             # iterative.py:483-490
        ap = a["aperture_mask"]
        aperture = ap if not isinstance(ap, (int, float, np.floating)) else np.float32(ap)
        probe_reg_weight = 0
    # the loss-and-gradient call exactly as iterative.py:524 makes it (smooth_rolloff_loss = 0)
    problem, geo, variant = objective.prepare(
        ns.obj, ns.probe, ns.positions, ns.positions_correction, ns.tilts, ns.tilts_correction,
        a["this_slice_distances"], a["edge_slice_thickness_multiplier"], a["measured_array"], a["algorithm_type"],
        a["this_wavelength"], update_probe, update_obj, update_pos, update_tilts, a["masks"],
        a["pixel_size_x_A"], a["pixel_size_y_A"], a["recon_type"], a["Cs"], a["defocus_array"],
        a["alpha_near_field"], a["damping_cutoff_multislice"], 0, a["propmethod"], a["this_chopped_sequence"],
        a["load_one_by_one"], a["data_multiplier"], a["data_pad"], a["phase_plate_in_h5"], a["this_loss_weight"],
        a["data_bin"], a["data_shift_vector"], a["upsample_pattern"], ns.static_background, update_sb, a["tilt_mode"],
        a["aberration_marker"], a["probe_marker"], ns.aberrations_array, a["compute_batch"], a["phase_only_obj"],
        ns.beam_current, update_bc, update_ab, a["default_float"], a["default_complex"], a["xp"], a["is_first_epoch"],
        a["scan_size"], a["scan_step_A"], a["fast_axis_reg_weight_positions"], a["slow_axis_reg_weight_positions"],
        a["slow_axis_reg_weight_tilts"], a["current_deformation_reg_weight_positions"],
        a["current_deformation_reg_weight_tilts"], a["fast_axis_reg_weight_tilts"], a["aperture_mask"],
        probe_reg_weight, a["current_window_weight"], a["current_window"], a["phase_norm_weight"],
        a["abs_norm_weight"], a["atv_weight"], a["atv_q"], a["atv_p"], a["mixed_variance_weight"],
        a["mixed_variance_sigma"], a["wedge_mu"], a["beta_wedge"], a["probe_mod_reg_weight"], a["probe_mod_tol"],
        a["smart_memory"], a["print_flag"], a["data_simulation_flag"], a["data_simulation_exitwave"],
        a["use_padded_intensity"])
    eng = default_engine()
    dev = eng.device
    if variant is not None:
        for k, dt in (("masks", torch.float32), ("beam_current", torch.float32), ("aberrations", torch.float32),
                      ("aberration_marker", torch.int32), ("static_background", torch.float32),
                      ("defocus_per_position", torch.float32), ("probe_marker", torch.int32)):
            if variant[k] is not None:
                variant[k] = _to_device(variant[k], dt, dev)
    st = _STATES.setdefault(id(ns), {"opt": None, "meas_src": None, "meas": None})
    meas_src = a["measured_array"]
    if st["meas_src"] is not meas_src:
        st["meas"] = objective.measured_tensor(meas_src, dev, bool(a["load_one_by_one"]))
        st["meas_src"] = meas_src
    obj_d = _to_device(ns.obj, torch.complex64, dev)
    probe_d = _to_device(ns.probe, torch.complex64, dev)
    corr_d = _to_device(ns.positions_correction, torch.float32, dev)
    cfg = LineSearchConfig(
        update_obj=update_obj, update_probe=update_probe, update_pos=update_pos,
        clean_cutoff=a["damping_cutoff_multislice"] - a["update_extra_cut"], smooth_rolloff=a["smooth_rolloff"],
        lazy_clean=bool(a["lazy_clean"]), keep_probe_states_orthogonal=bool(a["keep_probe_states_orthogonal"]),
        aperture=aperture, wolfe_c1=a["wolfe_c1_constant"], wolfe_c2=a["wolfe_c2_constant"],
        max_count=a["max_count"], reduce_factor=a["reduce_factor"], optimism=a["optimism"],
        stepsize_threshold_low=a["stepsize_threshold_low"], hist_length=int(a["hist_length"]),
        verbose=int(a["print_flag"] or 0), update_tilts=update_tilts, update_aberrations=update_ab,
        update_beam_current=update_bc, update_static_background=update_sb)
    # the variants path's extra variables: the tilt rows (without their correction), the refined
    # tilt correction, static background, aberration arrays and beam currents
    # (iterative.py:472-486)
    extras = dict(tilts=None, tilts_correction=None, aberrations=None, beam_current=None, static_background=None)
    if variant is not None:
        if variant.get("tilts") is not None:
            extras["tilts"] = _to_device(ns.tilts, torch.float32, dev)
            extras["tilts_correction"] = _to_device(ns.tilts_correction, torch.float32, dev)
        if variant.get("aberrations") is not None:
            extras["aberrations"] = variant["aberrations"]
        if variant.get("beam_current") is not None:
            extras["beam_current"] = variant["beam_current"]
        if variant.get("static_background") is not None:
            extras["static_background"] = variant["static_background"]
    opt = st["opt"]
    hist = getattr(ns, "history_bfgs", None)
    empty = hist is None or bool(hist.get("empty_hist", True))
    if opt is None or tuple(opt.obj.shape) != tuple(obj_d.shape) or tuple(opt.probe.shape) != tuple(probe_d.shape) \
            or tuple(opt.corr.shape) != tuple(corr_d.shape):
        opt = st["opt"] = LBFGS(problem, geo, st["meas"], obj_d, probe_d, corr_d, cfg, eng, variant=variant,
                                **extras)
    else:
        opt.problem, opt.geo, opt.measured, opt.cfg, opt.variant = problem, geo, st["meas"], cfg, variant
        opt.obj, opt.probe, opt.corr = obj_d, probe_d, corr_d
        opt.tilts, opt.tcorr, opt.ab, opt.bc = (extras["tilts"], extras["tilts_correction"], extras["aberrations"],
                                                extras["beam_current"])
        opt.sb = extras["static_background"]
    if empty:
        opt.reset()
    res = opt.step(a["actual_step"])
    warnings = a["warnings"] + "".join(res.warnings)
    counter_failed_epochs = a["counter_failed_epochs"]
    ns.obj = _like(opt.obj, ns.obj)
    ns.probe = _like(opt.probe, ns.probe)
    if res.accepted:
        counter_failed_epochs = 0
        if update_pos:
            ns.positions_correction = _like(opt.corr, ns.positions_correction)
        if update_tilts and opt.tcorr is not None:
            ns.tilts_correction = _like(opt.tcorr, ns.tilts_correction)
        if update_ab and opt.ab is not None:
            ns.aberrations_array = _like(opt.ab, ns.aberrations_array)
        if update_bc and opt.bc is not None:
            ns.beam_current = _like(opt.bc, ns.beam_current)
        if update_sb and opt.sb is not None:
            ns.static_background = _like(opt.sb, ns.static_background)
        h = ns.history_bfgs if isinstance(getattr(ns, "history_bfgs", None), dict) else _fresh_history()
        h["empty_hist"] = False
        h["prev_loss"], h["prev_sse"] = opt.prev[0], opt.prev[1]
        h["rho_hist"] = list(opt.history)        # device slots of the stored pairs, oldest first
        for k, v in opt.gammas().items():
            h["gamma_" + {"static_background": "static"}.get(k, k)] = v   # the reference's key names
        ns.history_bfgs = h
    else:
        counter_failed_epochs += 1
        if hasattr(ns, "reset_bfgs_history"):
            ns.reset_bfgs_history()
        else:
            ns.history_bfgs = _fresh_history()
        opt.reset()
    constraint_contributions = np.zeros(objective.N_CONSTRAINTS)
    return (res.total_loss, res.sse, constraint_contributions, res.actual_step, res.count, res.d_value,
            res.new_d_value, warnings, counter_failed_epochs)


def bfgs_update(algorithm_type, this_slice_distances, edge_slice_thickness_multiplier, this_step_probe,
                this_step_obj, this_step_pos_correction, this_step_tilts, measured_array, this_wavelength, masks,
                pixel_size_x_A, pixel_size_y_A, phase_norm_weight, abs_norm_weight, stepsize_threshold_low,
                probe_reg_weight, aperture_mask, recon_type, defocus_array, Cs, alpha_near_field,
                damping_cutoff_multislice, smooth_rolloff, update_extra_cut, keep_probe_states_orthogonal,
                do_charge_flip, cf_delta_phase, cf_delta_abs, cf_beta_phase, cf_beta_abs, phase_only_obj, wedge_mu,
                beta_wedge, wolfe_c1_constant, wolfe_c2_constant, atv_weight, atv_q, atv_p, tune_only_probe_phase,
                propmethod, this_chopped_sequence, load_one_by_one, data_multiplier, data_pad, phase_plate_in_h5,
                print_flag, this_loss_weight, max_count, reduce_factor, optimism, mixed_variance_weight,
                mixed_variance_sigma, data_bin, data_shift_vector, smart_memory, default_float, default_complex,
                default_int, upsample_pattern, this_step_static_background, tilt_mode, fancy_sigma,
                tune_only_probe_abs, aberration_marker, this_step_aberrations_array, probe_marker, compute_batch,
                current_window, current_window_weight, dynamically_resize_yx_object, lazy_clean,
                current_gaussian_filter, current_apply_gaussian_filter_amplitude, this_beam_current_step, xp,
                remove_fft_cache, is_first_epoch, hist_length, actual_step, fast_axis_reg_weight_positions,
                fast_axis_reg_weight_tilts, slow_axis_reg_weight_positions, slow_axis_reg_weight_tilts, scan_size,
                scan_step_A, current_deformation_reg_weight_positions, current_deformation_reg_weight_tilts,
                warnings, data_simulation_flag, data_simulation_exitwave, pos_puzzling, probe_mod_reg_weight,
                probe_mod_tol, use_padded_intensity, counter_failed_epochs):
    """One L-BFGS update with Wolfe line search of this module's ``obj`` / ``probe`` /
    ``positions_correction`` (``pypty/iterative.py:440-1049``). Returns (total_loss,
    this_sse, constraint_contributions, actual_step, count, d_value, new_d_value, warnings,
    counter_failed_epochs) like the reference."""
    return _impl(sys.modules[__name__], dict(locals()))


def bind(module):
    """``bfgs_update`` reading and writing the module variables of ``module`` (for
    example ``pypty.iterative``) instead of this module's."""
    sig = inspect.signature(bfgs_update)

    @functools.wraps(bfgs_update)
    def bound(*args, **kwargs):
        ba = sig.bind(*args, **kwargs)
        return _impl(module, dict(ba.arguments))

    return bound
