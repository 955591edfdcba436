"""Host-side logic of the drop-in: flag screening, geometry, problem construction."""
import numpy as np
import pytest

from pypty_gb300 import _lib, synth
from pypty_gb300.engine import Geometry, make_problem
from pypty_gb300 import objective


def base_kwargs(**over):
    W = 64
    kw = dict(this_obj=np.ones((96, 96, 1, 1), np.complex64), full_probe=np.ones((W, W, 1), np.complex64),
              this_pos_array=np.zeros((2, 2), np.int32), this_pos_correction=np.zeros((2, 2), np.float32),
              this_tilt_array=np.zeros((1, 6), np.float32), this_tilts_correction=np.zeros((1, 6), np.float32),
              this_distances=np.array([1.0], np.float32), edge_slice_thickness_multiplier=1.0,
              measured_array=np.zeros((2, W, W), np.float32), algorithm_type="lsq_sqrt",
              this_wavelength=np.float32(0.025), this_step_probe=1, this_step_obj=1,
              this_step_pos_correction=0, this_step_tilts=0, masks=None, pixel_size_x_A=0.2,
              pixel_size_y_A=0.2, recon_type="far_field", Cs=0, defocus_array=np.array([0.0]),
              alpha_near_field=0, damping_cutoff_multislice=2 / 3, smooth_rolloff=0,
              propmethod="multislice", this_chopped_sequence=np.arange(2), load_one_by_one=False,
              data_multiplier=1, data_pad=0, phase_plate_in_h5=None, this_loss_weight=1, data_bin=1,
              data_shift_vector=[0, 0], upsample_pattern=1, static_background=None,
              this_step_static_background=0, tilt_mode=0, aberration_marker=None, probe_marker=None,
              aberrations_array=None, compute_batch=2, phase_only_obj=False, beam_current=None,
              this_beam_current_step=0, this_step_aberrations_array=0, default_float=np.float32,
              default_complex=np.complex64, xp=np, is_first_epoch=True, scan_size=None, scan_step_A=1,
              fast_axis_reg_weight_positions=0, slow_axis_reg_weight_positions=0,
              slow_axis_reg_weight_tilts=0, current_deformation_reg_weight_positions=0,
              current_deformation_reg_weight_tilts=0, fast_axis_reg_weight_tilts=0, aperture_mask=None,
              probe_reg_weight=0, current_window_weight=0, current_window=None, phase_norm_weight=0,
              abs_norm_weight=0, atv_weight=0, atv_q=1, atv_p=2, mixed_variance_weight=0,
              mixed_variance_sigma=0.5, wedge_mu=0, beta_wedge=0, probe_mod_reg_weight=0,
              probe_mod_tol=0.05, smart_memory=False, print_flag=0, data_simulation_flag=False,
              data_simulation_exitwave=False, use_padded_intensity=True)
    kw.update(over)
    return kw


@pytest.mark.parametrize("over", [
    dict(recon_type="fresnel"), dict(recon_type="near_field", alpha_near_field=0.1),
    dict(recon_type="near_field", defocus_array=np.array([1.0, 2.0, 3.0])), dict(propmethod="yoshida"),
    dict(algorithm_type="lsq_compressed"), dict(algorithm_type="huber"),
    dict(tilt_mode=7), dict(this_tilt_array=np.ones((3, 6), np.float32)),
    dict(this_obj=np.ones((96, 96, 4, 1), np.complex64), this_distances=np.array([1.0, 2.0])), dict(phase_plate_in_h5="x.h5"),
    dict(full_probe=np.ones((64, 64, 1, 2), np.complex64)), dict(this_beam_current_step=1),
    dict(aberrations_array=np.zeros((1, 3), np.float32)), dict(data_bin=2),
    dict(algorithm_type="lsq_compressed", masks=np.ones((2, 64, 64), np.float32), data_pad=4),
    dict(upsample_pattern=2, algorithm_type="lsq_compressed", masks=np.ones((2, 64, 64), np.float32)),
    dict(atv_weight=0.1), dict(static_background=np.ones((64, 64)), upsample_pattern=2),
    dict(static_background=np.ones((64, 64)), data_pad=4, use_padded_intensity=False),
    dict(static_background=np.ones(64)), dict(this_step_static_background=1),
    dict(data_simulation_flag="sim.npy", data_bin=2),
])
def test_unsupported_flags_raise_before_any_gpu_work(over):
    with pytest.raises(NotImplementedError):
        objective.loss_and_direction(**base_kwargs(**over))


def test_reference_signature_is_mirrored():
    import inspect
    params = list(inspect.signature(objective.loss_and_direction).parameters)
    assert params[:4] == ["this_obj", "full_probe", "this_pos_array", "this_pos_correction"]
    assert len(params) == 77 and params[-1] == "use_padded_intensity"


def test_probe_shift_flag_follows_reference_rule():
    g = Geometry.make(np.zeros((3, 2)), np.zeros((3, 2)))
    assert not g.probe_shift(step_pos=False)
    assert g.probe_shift(step_pos=True)
    g = Geometry.make(np.zeros((3, 2)), np.array([[0, 0], [0.1, 0], [0, 0]]))
    assert g.probe_shift(step_pos=False)


def test_make_problem_fields():
    ipos, corr = synth.split_positions(synth.raster_positions(4, 4, 3.3))
    g = Geometry.make(ipos, corr)
    p = make_problem(128, (256, 256, 20, 1), 3, g, algorithm="ml", wavelength=0.0197,
                     pixel_size_x=0.1, pixel_size_y=0.1, slice_distance=2.0, compute_batch=8)
    assert (p.window, p.n_slices, p.n_probe_modes, p.n_positions, p.compute_batch) == (128, 20, 3, 16, 8)
    assert p.algorithm == _lib.ALGORITHMS["ml"] and p.probe_shift == 1
    assert abs(p.damping_cutoff - 2 / 3) < 1e-7


def test_split_positions_matches_reference_rounding():
    pos = np.array([[0.4, 1.6], [2.5, 3.49], [-1.2, 0.0]])
    ipos, corr = synth.split_positions(pos)
    shifted = pos - pos.min(axis=0)
    assert np.array_equal(ipos, np.round(shifted).astype(np.int32))
    assert np.allclose(corr, shifted - np.round(shifted), atol=1e-7)


def test_window_index_arrays_are_recognised_and_others_rejected():
    from pypty_gb300.multislice_core import _window_positions
    W = 64
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    pos = np.array([[3, 5], [10, 0]])
    my = pos[:, 0][:, None, None] + runy[None]
    mx = pos[:, 1][:, None, None] + runx[None]
    assert np.array_equal(_window_positions(my, mx, W), pos)
    with pytest.raises(NotImplementedError):
        _window_positions(my[:, ::-1], mx, W)


def test_bfgs_update_signature_is_mirrored():
    import inspect
    from pypty_gb300 import iterative
    params = list(inspect.signature(iterative.bfgs_update).parameters)
    assert len(params) == 95
    assert params[:4] == ["algorithm_type", "this_slice_distances", "edge_slice_thickness_multiplier",
                          "this_step_probe"]
    assert params[-1] == "counter_failed_epochs"
    assert params[params.index("hist_length") + 1] == "actual_step"
    bound = iterative.bind(object())
    assert list(inspect.signature(bound).parameters) == params


@pytest.mark.parametrize("flag", ["phase_only_obj", "tune_only_probe_phase", "this_step_static_background",
                                  "do_charge_flip", "current_gaussian_filter", "this_beam_current_step",
                                  "this_step_aberrations_array"])
def test_bfgs_update_unsupported_options_raise_before_any_gpu_work(flag):
    import inspect
    import types
    from pypty_gb300 import iterative
    ns = types.ModuleType("ns")
    ns.probe = np.zeros((64, 64, 1), np.complex64)
    kw = {p: 0 for p in inspect.signature(iterative.bfgs_update).parameters}
    kw.update(this_step_obj=1, this_step_probe=1, this_step_pos_correction=0, warnings="")
    kw[flag] = 1
    with pytest.raises(NotImplementedError):
        iterative.bind(ns)(**kw)


def test_variant_flags_route_to_the_variants_path():
    """Near field, compressed detectors, beam current, aberration plates and one inside tilt
    select pty_loss_and_direction_variants with the reference's values."""
    kw = base_kwargs(recon_type="near_field", defocus_array=np.array([55.0], np.float32), Cs=np.float32(2e5))
    _, _, v = objective.prepare(**kw)
    assert v["recon_type"] == "near_field" and v["defocus"] == 55.0 and v["cs"] == 2e5
    tilt = np.zeros((1, 6), np.float32)
    tilt[0, 2], tilt[0, 3] = -1e-3, 2e-3
    corr = np.zeros((1, 6), np.float32)
    corr[0, 3] = 1e-3
    _, _, v = objective.prepare(**base_kwargs(this_tilt_array=tilt, this_tilts_correction=corr))
    assert v["tilts"][0, 2] == pytest.approx(-1e-3) and v["tilts"][0, 3] == pytest.approx(3e-3)   # + correction
    rows = np.full((2, 6), 1e-3, np.float32)
    _, _, v = objective.prepare(**base_kwargs(this_tilt_array=rows, this_tilts_correction=np.zeros_like(rows),
                                              tilt_mode=4, this_step_tilts=1))
    assert v["tilt_mode"] == 4 and v["step_tilts"] and v["tilts"].shape == (2, 6)
    masks = np.ones((3, 64, 64), np.float32)
    _, _, v = objective.prepare(**base_kwargs(algorithm_type="poisson_compressed", masks=masks,
                                              measured_array=np.zeros((2, 3), np.float32)))
    assert v["masks"].shape == (3, 64, 64)
    _, _, v = objective.prepare(**base_kwargs(beam_current=np.ones(2, np.float32), this_beam_current_step=1,
                                              aberrations_array=np.zeros((1, 4), np.float32),
                                              aberration_marker=np.zeros(2, int), this_step_aberrations_array=1))
    assert v["step_beam_current"] and v["step_aberrations"] and v["aberrations"].shape == (1, 4)
    p, _, v = objective.prepare(**base_kwargs())
    assert v is None and p.algorithm == _lib.ALGORITHMS["lsq_sqrt"]


def test_measured_preprocessing_routes_to_the_variants_path():
    _, _, v = objective.prepare(**base_kwargs(data_pad=4, use_padded_intensity=False,
                                              measured_array=np.zeros((2, 56, 56), np.float32)))
    assert v["data_pad"] == 4 and v["use_padded_intensity"] is False
    _, _, v = objective.prepare(**base_kwargs(data_shift_vector=[1, -2], data_multiplier=2.0))
    assert v["data_shift_vector"] == (1, -2) and v["data_multiplier"] == 2.0


def test_upsampling_and_static_background_route_to_the_variants_path():
    """upsample_pattern and a 2D static background (with its step) select the variants path;
    a scalar zero background is no background."""
    _, _, v = objective.prepare(**base_kwargs(upsample_pattern=2, measured_array=np.zeros((2, 32, 32), np.float32)))
    assert v["upsample_pattern"] == 2 and v["static_background"] is None
    bg = np.full((64, 64), 0.5, np.float32)
    _, _, v = objective.prepare(**base_kwargs(static_background=bg, this_step_static_background=1))
    assert v["static_background"].shape == (64, 64) and v["step_static_background"]
    _, _, v = objective.prepare(**base_kwargs(static_background=0))
    assert v is None


def test_per_slice_distances_reach_the_problem():
    """this_distances with one entry per slice step is passed to the C ABI (slice_distances);
    one entry keeps the single-distance tables."""
    obj = np.ones((96, 96, 4, 1), np.complex64)
    p, _, v = objective.prepare(**base_kwargs(this_obj=obj, this_distances=np.array([1.0, 2.0, 3.0], np.float32)))
    assert v is None and p.slice_distances
    assert list(p._slice_distances) == [1.0, 2.0, 3.0] and p.slice_distance == 1.0
    p, _, _ = objective.prepare(**base_kwargs(this_obj=obj, this_distances=np.array([2.0], np.float32)))
    assert not p.slice_distances and p.slice_distance == 2.0


def test_per_position_defocus_routes_to_the_variants_path():
    _, _, v = objective.prepare(**base_kwargs(recon_type="near_field", defocus_array=np.array([10.0, 20.0])))
    assert v["defocus"] == 10.0 and list(v["defocus_per_position"]) == [10.0, 20.0]
    _, _, v = objective.prepare(**base_kwargs(recon_type="near_field", defocus_array=np.array([10.0])))
    assert v["defocus_per_position"] is None


def test_probe_scenarios_route_to_the_variants_path():
    """A 4D probe with probe_marker selects the variants path; a marker with a 3D probe is
    ignored, as the reference ignores it (multiple_scenarios needs both, objective.py:285)."""
    probe = np.ones((64, 64, 1, 3), np.complex64)
    _, _, v = objective.prepare(**base_kwargs(full_probe=probe, probe_marker=np.array([0, 2])))
    assert list(v["probe_marker"]) == [0, 2]
    _, _, v = objective.prepare(**base_kwargs(probe_marker=np.array([0, 1])))
    assert v is None


def test_complex128_request_warns_once_and_names_complex64():
    """The reference's default dtype is "double" (pypty/iterative.py:58-60); the GPU path
    computes in complex64 and says so instead of narrowing silently."""
    import warnings
    kw = base_kwargs(this_obj=np.ones((96, 96, 1, 1), np.complex128),
                     full_probe=np.ones((64, 64, 1), np.complex128), default_complex=np.complex128,
                     default_float=np.float64)
    with pytest.warns(objective.ComputePrecisionWarning, match="complex64"):
        objective.prepare(**kw)
    with warnings.catch_warnings():
        warnings.simplefilter("error", objective.ComputePrecisionWarning)
        objective.prepare(**base_kwargs())          # complex64 throughout: no warning
    with pytest.warns(objective.ComputePrecisionWarning):
        objective.prepare(**base_kwargs(default_complex=np.complex128))   # the dtype argument alone


def test_duplicate_sequence_entries_keep_the_last_position_gradient_rule():
    """finalize_scalars_kernel writes pos_grad[seq[i]] only for the last occurrence of a
    position in the sequence; this restates that selection on the host for a sequence with
    repeats inside one round of 256 entries and across rounds."""
    rng = np.random.default_rng(0)
    seq = rng.integers(0, 40, 700)
    writer = {}
    for base in range(0, len(seq), 256):
        r = seq[base:base + 256]
        for k, s in enumerate(r):
            if not np.any(r[k + 1:] == s):
                writer[int(s)] = base + k
    last = {int(s): i for i, s in enumerate(seq)}
    assert writer == last
