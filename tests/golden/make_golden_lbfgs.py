"""Golden vectors of the optimizer step, from the reference's own NumPy path.

Run where the reference sources are mounted (``PYPTY_REFERENCE_ROOT`` names the
reference checkout; it is required)::

    python tests/golden/make_golden_lbfgs.py [clean lbfgs refine static scenarios]   # all without names

* ``fourier_clean_c64.npz``: ``pypty.utils.fourier_clean`` (``pypty/utils.py:102``) on 2D,
  3D and 4D complex64 arrays with and without a cosine roll-off and with a given mask.
* ``lbfgs_<case>.npz``: several consecutive calls of ``pypty.iterative.bfgs_update``
  (``pypty/iterative.py:440``) on the module variables ``obj``, ``probe``,
  ``positions_correction``, starting from an empty history; the returned scalars of every
  call and the arrays after every call.
* ``lbfgs_refine_tilts_aberr_current.npz`` / ``lbfgs_refine_static_background.npz``: the same
  with tilt corrections, aberration arrays and beam currents, or the static background,
  refined together with the object and probe.
* ``lbfgs_refine_probe_scenarios.npz``: two probe scenarios (a 4D probe with probe_marker),
  modes kept orthogonal.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from refimport import import_reference  # noqa: E402
from pypty_gb300 import synth  # noqa: E402
from make_golden import build_case  # noqa: E402


def make_clean_case(pypty):
    rng = np.random.default_rng(21)
    f = np.float32
    out = {}
    shapes = [("a2", (64, 128), f(0.66), f(0)), ("a3", (128, 64, 3), f(2 / 3) - f(0.005), f(0.1)),
              ("a4", (64, 64, 3, 2), f(2 / 3) - f(0.005), f(0)), ("a4r", (64, 64, 2, 2), f(0.5), f(0.2))]
    for name, shape, cutoff, rolloff in shapes:
        a = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)
        res = pypty.utils.fourier_clean(a.copy(), cutoff=cutoff, rolloff=rolloff, default_float=f, xp=np)
        out[name + "_in"] = a
        out[name + "_cut"] = np.array([cutoff, rolloff], dtype=np.float32)
        out[name + "_out"] = np.asarray(res)
    # a given (fftshifted) aperture mask
    a = (rng.normal(size=(64, 64, 2)) + 1j * rng.normal(size=(64, 64, 2))).astype(np.complex64)
    yy, xx = np.mgrid[:64, :64]
    mask = (((yy - 32) ** 2 + (xx - 32) ** 2) < 15 ** 2).astype(np.float32)
    res = pypty.utils.fourier_clean(a.copy(), mask=mask, default_float=f, xp=np)
    out["m_in"], out["m_mask"], out["m_out"] = a, mask, np.asarray(res)
    path = os.path.join(HERE, "fourier_clean_c64.npz")
    np.savez_compressed(path, **out)
    print("fourier_clean -> %s" % path)


def ref_bfgs_epochs(pypty, c, n_epochs, opts):
    """Drive pypty.iterative.bfgs_update with every argument spelled out (iterative.py:440)."""
    it = pypty.iterative
    f, cx = np.float32, np.complex64
    it.obj = c["obj"].copy()
    it.probe = c["probe"].copy()
    it.positions = c["positions"].copy()
    it.positions_correction = c["pos_correction"].astype(f).copy()
    it.tilts = np.zeros((1, 6), dtype=f)
    it.tilts_correction = np.zeros((1, 6), dtype=f)
    it.static_background = None
    it.aberrations_array = None
    it.beam_current = None
    it.reset_bfgs_history()
    np.random.seed(5)
    rec = dict(scalars=[], obj=[], probe=[], corr=[])
    warnings, failed = "", 0
    for epoch in range(n_epochs):
        res = it.bfgs_update(
            algorithm_type=c["algorithm"], this_slice_distances=np.array([c["distance"]], dtype=f),
            edge_slice_thickness_multiplier=c["edge_mult"], this_step_probe=opts["step_probe"],
            this_step_obj=opts["step_obj"], this_step_pos_correction=opts["step_pos"], this_step_tilts=0,
            measured_array=c["measured"], this_wavelength=f(c["wavelength"]), masks=None,
            pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]), phase_norm_weight=0, abs_norm_weight=0,
            stepsize_threshold_low=1e-20, probe_reg_weight=0, aperture_mask=None, recon_type="far_field",
            defocus_array=np.array([0.0], dtype=f), Cs=f(0), alpha_near_field=f(0),
            damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(opts["rolloff"]),
            update_extra_cut=f(0.005), keep_probe_states_orthogonal=opts["orthogonal"], do_charge_flip=False,
            cf_delta_phase=0, cf_delta_abs=0, cf_beta_phase=0, cf_beta_abs=0, phase_only_obj=False, wedge_mu=0,
            beta_wedge=0, wolfe_c1_constant=0.1, wolfe_c2_constant=0.9, atv_weight=0, atv_q=1, atv_p=2,
            tune_only_probe_phase=False, propmethod="multislice", this_chopped_sequence=c["sequence"],
            load_one_by_one=False, data_multiplier=f(1), data_pad=0, phase_plate_in_h5=None, print_flag=0,
            this_loss_weight=c["loss_weight"], max_count=20, reduce_factor=f(0.1), optimism=3,
            mixed_variance_weight=0, mixed_variance_sigma=0.5, data_bin=1, data_shift_vector=[0, 0],
            smart_memory=opts["smart_memory"], default_float=f, default_complex=cx, default_int=np.int32,
            upsample_pattern=1, this_step_static_background=0, tilt_mode=0, fancy_sigma=None,
            tune_only_probe_abs=False, aberration_marker=None, this_step_aberrations_array=0, probe_marker=None,
            compute_batch=c["batch"], current_window=None, current_window_weight=0,
            dynamically_resize_yx_object=False, lazy_clean=opts["lazy_clean"], current_gaussian_filter=False,
            current_apply_gaussian_filter_amplitude=False, this_beam_current_step=0, xp=np,
            remove_fft_cache=False, is_first_epoch=epoch == 0, hist_length=opts["hist_length"], actual_step=1,
            fast_axis_reg_weight_positions=0, fast_axis_reg_weight_tilts=0, slow_axis_reg_weight_positions=0,
            slow_axis_reg_weight_tilts=0, scan_size=None, scan_step_A=1,
            current_deformation_reg_weight_positions=0, current_deformation_reg_weight_tilts=0,
            warnings=warnings, data_simulation_flag=False, data_simulation_exitwave=False, pos_puzzling=False,
            probe_mod_reg_weight=0, probe_mod_tol=0.05, use_padded_intensity=True, counter_failed_epochs=failed)
        total_loss, sse, _cc, actual_step, count, d_value, new_d_value, warnings, failed = res
        rec["scalars"].append([float(total_loss), float(sse), float(actual_step), float(count), float(d_value),
                               float(new_d_value), float(failed)])
        rec["obj"].append(np.asarray(it.obj).copy())
        rec["probe"].append(np.asarray(it.probe).copy())
        rec["corr"].append(np.asarray(it.positions_correction).copy())
    return rec


CASES = [
    # object + probe, Poisson loss, two probe modes, one slice distance, four calls (history 3)
    ("obj_probe_ml", dict(seed=31, W=64, ny=128, nx=128, Z=2, Mo=1, Mp=2, n_scan=5, step_px=10.0,
                          jitter_px=1.0, algorithm="ml", batch=25, px=0.1, kV=300.0, alpha=30.0, defocus=40.0,
                          distance=2.0, dose=1e5),
     dict(step_obj=1, step_probe=1, step_pos=0, rolloff=0.0, orthogonal=False, smart_memory=False,
          lazy_clean=False, hist_length=10), 4),
    # position corrections too, amplitude loss, hist_length 2 (history trimmed)
    ("pos_lsq_sqrt", dict(seed=32, W=64, ny=128, nx=128, Z=1, Mo=1, Mp=1, n_scan=5, step_px=10.0,
                          jitter_px=1.5, algorithm="lsq_sqrt", batch=13, px=0.2, dose=1e4),
     dict(step_obj=1, step_probe=1, step_pos=1, rolloff=0.0, orthogonal=False, smart_memory=True,
          lazy_clean=False, hist_length=2), 4),
    # roll-off, orthogonalised probe modes, lazy clean
    ("rolloff_orth_lazy", dict(seed=33, W=64, ny=128, nx=128, Z=2, Mo=1, Mp=3, n_scan=4, step_px=12.0,
                               jitter_px=1.0, algorithm="lsq_sqrt", batch=16, px=0.15, dose=1e4),
     dict(step_obj=1, step_probe=1, step_pos=0, rolloff=0.1, orthogonal=True, smart_memory=False,
          lazy_clean=True, hist_length=10), 3),
]


def make_lbfgs_cases(pypty):
    for name, spec, opts, n_epochs in CASES:
        c = build_case(name, **spec)
        rec = ref_bfgs_epochs(pypty, c, n_epochs, opts)
        path = os.path.join(HERE, "lbfgs_%s.npz" % name)
        np.savez_compressed(
            path, obj=c["obj"], probe=c["probe"], positions=c["positions"], pos_correction=c["pos_correction"],
            measured=c["measured"], sequence=c["sequence"],
            scalars=np.array([c["distance"], c["edge_mult"], c["wavelength"], c["px"], c["cutoff"], c["rolloff"],
                              c["loss_weight"], c["batch"]], dtype=np.float64),
            algorithm=np.array(c["algorithm"]),
            opts=np.array([opts["step_obj"], opts["step_probe"], opts["step_pos"], opts["rolloff"],
                           opts["orthogonal"], opts["smart_memory"], opts["lazy_clean"], opts["hist_length"]],
                          dtype=np.float64),
            ref_scalars=np.array(rec["scalars"]), ref_obj=np.stack(rec["obj"]), ref_probe=np.stack(rec["probe"]),
            ref_corr=np.stack(rec["corr"]))
        print("%-20s %s -> %s" % (name, " ".join("%.5g/%d" % (s[0], s[3]) for s in rec["scalars"]), path))


def make_refine_case(pypty):
    """``lbfgs_refine_tilts_aberr_current.npz``: object, probe, per-position tilt corrections
    (tilt_mode 3), aberration arrays and beam currents refined together by three calls of
    ``bfgs_update`` (``pypty/iterative.py:477-481, 562-672, 869-916``)."""
    it = pypty.iterative
    f, cx = np.float32, np.complex64
    c = build_case("refine", seed=36, W=64, ny=128, nx=128, Z=2, Mo=1, Mp=2, n_scan=5, step_px=8.0, jitter_px=0.0,
                   algorithm="ml", batch=10, px=0.15, kV=300.0, alpha=30.0, defocus=40.0, distance=2.0, dose=1e5,
                   integer_positions=True)
    rng = np.random.default_rng(77)
    N = c["positions"].shape[0]
    tilts = (rng.normal(size=(N, 6)) * 3e-4).astype(f)
    bc = (1.0 + 0.1 * rng.normal(size=N)).astype(f)
    ab = (rng.normal(size=(2, 4)) * 10.0).astype(f)
    marker = (np.arange(N) % 2).astype(np.int64)
    it.obj, it.probe = c["obj"].copy(), c["probe"].copy()
    it.positions = c["positions"].copy()
    it.positions_correction = c["pos_correction"].astype(f).copy()
    it.tilts, it.tilts_correction = tilts.copy(), np.zeros_like(tilts)
    it.static_background = None
    it.aberrations_array, it.beam_current = ab.copy(), bc.copy()
    it.reset_bfgs_history()
    np.random.seed(5)
    rec = dict(scalars=[], obj=[], probe=[], tcorr=[], ab=[], bc=[])
    warnings, failed = "", 0
    # a float first step (with the integer 1 a random-step trial truncates to 0, iterative.py:831),
    # small enough that the Wolfe search settles without random trial steps: a sequence that
    # draws random steps flips with any rounding difference
    step = 1e-3
    for epoch in range(3):
        res = it.bfgs_update(
            algorithm_type=c["algorithm"], this_slice_distances=np.array([c["distance"]], dtype=f),
            edge_slice_thickness_multiplier=c["edge_mult"], this_step_probe=1, this_step_obj=1,
            this_step_pos_correction=0, this_step_tilts=1, measured_array=c["measured"],
            this_wavelength=f(c["wavelength"]), masks=None, pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]),
            phase_norm_weight=0, abs_norm_weight=0, stepsize_threshold_low=1e-20, probe_reg_weight=0,
            aperture_mask=None, recon_type="far_field", defocus_array=np.array([0.0], dtype=f), Cs=f(0),
            alpha_near_field=f(0), damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(0),
            update_extra_cut=f(0.005), keep_probe_states_orthogonal=False, do_charge_flip=False, cf_delta_phase=0,
            cf_delta_abs=0, cf_beta_phase=0, cf_beta_abs=0, phase_only_obj=False, wedge_mu=0, beta_wedge=0,
            wolfe_c1_constant=0.1, wolfe_c2_constant=0.9, atv_weight=0, atv_q=1, atv_p=2,
            tune_only_probe_phase=False, propmethod="multislice", this_chopped_sequence=c["sequence"],
            load_one_by_one=False, data_multiplier=f(1), data_pad=0, phase_plate_in_h5=None, print_flag=0,
            this_loss_weight=c["loss_weight"], max_count=20, reduce_factor=f(0.1), optimism=3,
            mixed_variance_weight=0, mixed_variance_sigma=0.5, data_bin=1, data_shift_vector=[0, 0],
            smart_memory=False, default_float=f, default_complex=cx, default_int=np.int32, upsample_pattern=1,
            this_step_static_background=0, tilt_mode=3, fancy_sigma=None, tune_only_probe_abs=False,
            aberration_marker=marker, this_step_aberrations_array=1, probe_marker=None,
            compute_batch=c["batch"], current_window=None, current_window_weight=0,
            dynamically_resize_yx_object=False, lazy_clean=False, current_gaussian_filter=False,
            current_apply_gaussian_filter_amplitude=False, this_beam_current_step=1, xp=np,
            remove_fft_cache=False, is_first_epoch=epoch == 0, hist_length=10, actual_step=step,
            fast_axis_reg_weight_positions=0, fast_axis_reg_weight_tilts=0, slow_axis_reg_weight_positions=0,
            slow_axis_reg_weight_tilts=0, scan_size=None, scan_step_A=1,
            current_deformation_reg_weight_positions=0, current_deformation_reg_weight_tilts=0,
            warnings=warnings, data_simulation_flag=False, data_simulation_exitwave=False, pos_puzzling=False,
            probe_mod_reg_weight=0, probe_mod_tol=0.05, use_padded_intensity=True, counter_failed_epochs=failed)
        total_loss, sse, _cc, actual_step, count, d_value, new_d_value, warnings, failed = res
        step = actual_step        # the next call starts from the accepted step, as run does
        rec["scalars"].append([float(total_loss), float(sse), float(actual_step), float(count), float(d_value),
                               float(new_d_value), float(failed)])
        rec["obj"].append(np.asarray(it.obj).copy())
        rec["probe"].append(np.asarray(it.probe).copy())
        rec["tcorr"].append(np.asarray(it.tilts_correction).copy())
        rec["ab"].append(np.asarray(it.aberrations_array).copy())
        rec["bc"].append(np.asarray(it.beam_current).copy())
    path = os.path.join(HERE, "lbfgs_refine_tilts_aberr_current.npz")
    np.savez_compressed(
        path, obj=c["obj"], probe=c["probe"], positions=c["positions"], pos_correction=c["pos_correction"],
        measured=c["measured"], sequence=c["sequence"], tilts=tilts, beam_current=bc, aberrations=ab,
        aberration_marker=marker,
        scalars=np.array([c["distance"], c["edge_mult"], c["wavelength"], c["px"], c["cutoff"], c["rolloff"],
                          c["loss_weight"], c["batch"]], dtype=np.float64),
        algorithm=np.array(c["algorithm"]), ref_scalars=np.array(rec["scalars"]), ref_obj=np.stack(rec["obj"]),
        ref_probe=np.stack(rec["probe"]), ref_tcorr=np.stack(rec["tcorr"]), ref_ab=np.stack(rec["ab"]),
        ref_bc=np.stack(rec["bc"]))
    print("refine %s -> %s" % (" ".join("%.5g/%d" % (s[0], s[3]) for s in rec["scalars"]), path))


def make_static_case(pypty):
    """Object, probe and static background refined together (iterative.py:569-916 with
    update_static_background): three bfgs_update calls of the reference, the static background
    after every call."""
    it = pypty.iterative
    f, cx = np.float32, np.complex64
    c = build_case("static", seed=37, W=64, ny=128, nx=128, Z=2, Mo=1, Mp=2, n_scan=5, step_px=8.0, jitter_px=0.0,
                   algorithm="lsq_sqrt", batch=10, px=0.15, kV=300.0, alpha=30.0, defocus=40.0, distance=2.0,
                   dose=1e5, integer_positions=True)
    rng = np.random.default_rng(78)
    W = c["probe"].shape[0]
    sb = (0.5 * np.sqrt(1e5 / (W * W)) * rng.uniform(0.5, 1.5, size=(W, W))).astype(f)
    it.obj, it.probe = c["obj"].copy(), c["probe"].copy()
    it.positions = c["positions"].copy()
    it.positions_correction = c["pos_correction"].astype(f).copy()
    it.tilts = np.zeros((1, 6), f)
    it.tilts_correction = np.zeros((1, 6), f)
    it.static_background = sb.copy()
    it.aberrations_array, it.beam_current = None, None
    it.reset_bfgs_history()
    np.random.seed(6)
    rec = dict(scalars=[], obj=[], probe=[], sb=[])
    warnings, failed = "", 0
    step = 1.0
    for epoch in range(3):
        res = it.bfgs_update(
            algorithm_type=c["algorithm"], this_slice_distances=np.array([c["distance"]], dtype=f),
            edge_slice_thickness_multiplier=c["edge_mult"], this_step_probe=1, this_step_obj=1,
            this_step_pos_correction=0, this_step_tilts=0, measured_array=c["measured"],
            this_wavelength=f(c["wavelength"]), masks=None, pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]),
            phase_norm_weight=0, abs_norm_weight=0, stepsize_threshold_low=1e-20, probe_reg_weight=0,
            aperture_mask=None, recon_type="far_field", defocus_array=np.array([0.0], dtype=f), Cs=f(0),
            alpha_near_field=f(0), damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(0),
            update_extra_cut=f(0.005), keep_probe_states_orthogonal=False, do_charge_flip=False, cf_delta_phase=0,
            cf_delta_abs=0, cf_beta_phase=0, cf_beta_abs=0, phase_only_obj=False, wedge_mu=0, beta_wedge=0,
            wolfe_c1_constant=0.1, wolfe_c2_constant=0.9, atv_weight=0, atv_q=1, atv_p=2,
            tune_only_probe_phase=False, propmethod="multislice", this_chopped_sequence=c["sequence"],
            load_one_by_one=False, data_multiplier=f(1), data_pad=0, phase_plate_in_h5=None, print_flag=0,
            this_loss_weight=c["loss_weight"], max_count=20, reduce_factor=f(0.1), optimism=3,
            mixed_variance_weight=0, mixed_variance_sigma=0.5, data_bin=1, data_shift_vector=[0, 0],
            smart_memory=False, default_float=f, default_complex=cx, default_int=np.int32, upsample_pattern=1,
            this_step_static_background=1, tilt_mode=0, fancy_sigma=None, tune_only_probe_abs=False,
            aberration_marker=None, this_step_aberrations_array=0, probe_marker=None,
            compute_batch=c["batch"], current_window=None, current_window_weight=0,
            dynamically_resize_yx_object=False, lazy_clean=False, current_gaussian_filter=False,
            current_apply_gaussian_filter_amplitude=False, this_beam_current_step=0, xp=np,
            remove_fft_cache=False, is_first_epoch=epoch == 0, hist_length=10, actual_step=step,
            fast_axis_reg_weight_positions=0, fast_axis_reg_weight_tilts=0, slow_axis_reg_weight_positions=0,
            slow_axis_reg_weight_tilts=0, scan_size=None, scan_step_A=1,
            current_deformation_reg_weight_positions=0, current_deformation_reg_weight_tilts=0,
            warnings=warnings, data_simulation_flag=False, data_simulation_exitwave=False, pos_puzzling=False,
            probe_mod_reg_weight=0, probe_mod_tol=0.05, use_padded_intensity=True, counter_failed_epochs=failed)
        total_loss, sse, _cc, actual_step, count, d_value, new_d_value, warnings, failed = res
        step = actual_step
        rec["scalars"].append([float(total_loss), float(sse), float(actual_step), float(count), float(d_value),
                               float(new_d_value), float(failed)])
        rec["obj"].append(np.asarray(it.obj).copy())
        rec["probe"].append(np.asarray(it.probe).copy())
        rec["sb"].append(np.asarray(it.static_background).copy())
    path = os.path.join(HERE, "lbfgs_refine_static_background.npz")
    np.savez_compressed(
        path, obj=c["obj"], probe=c["probe"], positions=c["positions"], pos_correction=c["pos_correction"],
        measured=c["measured"], sequence=c["sequence"], static_background=sb,
        scalars=np.array([c["distance"], c["edge_mult"], c["wavelength"], c["px"], c["cutoff"], c["rolloff"],
                          c["loss_weight"], c["batch"]], dtype=np.float64),
        algorithm=np.array(c["algorithm"]), ref_scalars=np.array(rec["scalars"]), ref_obj=np.stack(rec["obj"]),
        ref_probe=np.stack(rec["probe"]), ref_sb=np.stack(rec["sb"]))
    print("static %s -> %s" % (" ".join("%.5g/%d" % (s[0], s[3]) for s in rec["scalars"]), path))


def make_scenario_case(pypty):
    """Two probe scenarios (a 4D probe with probe_marker) with two modes each, kept orthogonal
    (keep_probe_states_orthogonal, objective.py:1119-1141 as bfgs_update calls it): three
    bfgs_update calls of the reference, object and probe after every call."""
    it = pypty.iterative
    f, cx = np.float32, np.complex64
    c = build_case("scenarios", seed=38, W=64, ny=128, nx=128, Z=2, Mo=1, Mp=2, n_scan=5, step_px=8.0,
                   jitter_px=1.0, algorithm="ml", batch=10, px=0.15, kV=300.0, alpha=30.0, defocus=40.0,
                   distance=2.0, dose=1e5)
    W = c["probe"].shape[0]
    probe2 = synth.make_probe(W, 0.15, 300.0, 30.0, 70.0, 2, [0.5, 0.3], 1e5, dtype=cx)
    probe4 = np.stack([c["probe"], probe2], -1)                     # (W, W, Mp, S)
    N = c["positions"].shape[0]
    marker = (np.arange(N) % 2).astype(np.int64)
    it.obj, it.probe = c["obj"].copy(), probe4.copy()
    it.positions = c["positions"].copy()
    it.positions_correction = c["pos_correction"].astype(f).copy()
    it.tilts = np.zeros((1, 6), f)
    it.tilts_correction = np.zeros((1, 6), f)
    it.static_background = None
    it.aberrations_array, it.beam_current = None, None
    it.reset_bfgs_history()
    np.random.seed(7)
    rec = dict(scalars=[], obj=[], probe=[])
    warnings, failed = "", 0
    step = 1.0
    for epoch in range(3):
        res = it.bfgs_update(
            algorithm_type=c["algorithm"], this_slice_distances=np.array([c["distance"]], dtype=f),
            edge_slice_thickness_multiplier=c["edge_mult"], this_step_probe=1, this_step_obj=1,
            this_step_pos_correction=0, this_step_tilts=0, measured_array=c["measured"],
            this_wavelength=f(c["wavelength"]), masks=None, pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]),
            phase_norm_weight=0, abs_norm_weight=0, stepsize_threshold_low=1e-20, probe_reg_weight=0,
            aperture_mask=None, recon_type="far_field", defocus_array=np.array([0.0], dtype=f), Cs=f(0),
            alpha_near_field=f(0), damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(0),
            update_extra_cut=f(0.005), keep_probe_states_orthogonal=True, do_charge_flip=False, cf_delta_phase=0,
            cf_delta_abs=0, cf_beta_phase=0, cf_beta_abs=0, phase_only_obj=False, wedge_mu=0, beta_wedge=0,
            wolfe_c1_constant=0.1, wolfe_c2_constant=0.9, atv_weight=0, atv_q=1, atv_p=2,
            tune_only_probe_phase=False, propmethod="multislice", this_chopped_sequence=c["sequence"],
            load_one_by_one=False, data_multiplier=f(1), data_pad=0, phase_plate_in_h5=None, print_flag=0,
            this_loss_weight=c["loss_weight"], max_count=20, reduce_factor=f(0.1), optimism=3,
            mixed_variance_weight=0, mixed_variance_sigma=0.5, data_bin=1, data_shift_vector=[0, 0],
            smart_memory=False, default_float=f, default_complex=cx, default_int=np.int32, upsample_pattern=1,
            this_step_static_background=0, tilt_mode=0, fancy_sigma=None, tune_only_probe_abs=False,
            aberration_marker=None, this_step_aberrations_array=0, probe_marker=marker,
            compute_batch=c["batch"], current_window=None, current_window_weight=0,
            dynamically_resize_yx_object=False, lazy_clean=False, current_gaussian_filter=False,
            current_apply_gaussian_filter_amplitude=False, this_beam_current_step=0, xp=np,
            remove_fft_cache=False, is_first_epoch=epoch == 0, hist_length=10, actual_step=step,
            fast_axis_reg_weight_positions=0, fast_axis_reg_weight_tilts=0, slow_axis_reg_weight_positions=0,
            slow_axis_reg_weight_tilts=0, scan_size=None, scan_step_A=1,
            current_deformation_reg_weight_positions=0, current_deformation_reg_weight_tilts=0,
            warnings=warnings, data_simulation_flag=False, data_simulation_exitwave=False, pos_puzzling=False,
            probe_mod_reg_weight=0, probe_mod_tol=0.05, use_padded_intensity=True, counter_failed_epochs=failed)
        total_loss, sse, _cc, actual_step, count, d_value, new_d_value, warnings, failed = res
        step = actual_step
        rec["scalars"].append([float(total_loss), float(sse), float(actual_step), float(count), float(d_value),
                               float(new_d_value), float(failed)])
        rec["obj"].append(np.asarray(it.obj).copy())
        rec["probe"].append(np.asarray(it.probe).copy())
    path = os.path.join(HERE, "lbfgs_refine_probe_scenarios.npz")
    np.savez_compressed(
        path, obj=c["obj"], probe=probe4, positions=c["positions"], pos_correction=c["pos_correction"],
        measured=c["measured"], sequence=c["sequence"], probe_marker=marker,
        scalars=np.array([c["distance"], c["edge_mult"], c["wavelength"], c["px"], c["cutoff"], c["rolloff"],
                          c["loss_weight"], c["batch"]], dtype=np.float64),
        algorithm=np.array(c["algorithm"]), ref_scalars=np.array(rec["scalars"]), ref_obj=np.stack(rec["obj"]),
        ref_probe=np.stack(rec["probe"]))
    print("scenarios %s -> %s" % (" ".join("%.5g/%d" % (s[0], s[3]) for s in rec["scalars"]), path))


if __name__ == "__main__":
    pypty = import_reference()
    from pypty import iterative  # noqa: F401
    makers = dict(clean=make_clean_case, lbfgs=make_lbfgs_cases, refine=make_refine_case, static=make_static_case,
                  scenarios=make_scenario_case)
    for name in sys.argv[1:] or list(makers):
        makers[name](pypty)
