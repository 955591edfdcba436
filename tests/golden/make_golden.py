"""Generate golden vectors by running the reference's own NumPy path.

Run where the reference sources are mounted (``PYPTY_REFERENCE_ROOT`` names the
reference checkout; it is required)::

    python tests/golden/make_golden.py [case names]   # every case and the core case without names

For every case it builds seeded inputs (``pypty_gb300.synth``), simulates measured
patterns with the oracle's forward model plus Poisson noise, evaluates the reference's
``pypty.objective.loss_and_direction`` (``pypty/objective.py:47``) at a perturbed
object/probe, and writes inputs and outputs to ``tests/golden/<case>.npz``. A second set
calls ``pypty.multislice_core.multislice`` / ``multislice_grads`` / ``scatteradd``
directly (``pypty/multislice_core.py:9,85,206``).
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
from oracle import ptycho_oracle as orc  # noqa: E402


def ref_loss_and_direction(pypty, c, obj, probe):
    """Call the reference with every argument spelled out (signature objective.py:47)."""
    f, cx = (np.float64, np.complex128) if c["double"] else (np.float32, np.complex64)
    N = c["positions"].shape[0]
    tilts = np.zeros((1, 6), dtype=f)
    res = pypty.objective.loss_and_direction(
        this_obj=obj.astype(cx), full_probe=probe.astype(cx),
        this_pos_array=c["positions"].copy(), this_pos_correction=c["pos_correction"].astype(f),
        this_tilt_array=tilts, this_tilts_correction=np.zeros_like(tilts),
        this_distances=(np.array([c["distance"]], dtype=f) if c.get("distances") is None
                        else np.asarray(c["distances"], dtype=f)),
        edge_slice_thickness_multiplier=c["edge_mult"], measured_array=c["measured"],
        algorithm_type=c["algorithm"], this_wavelength=f(c["wavelength"]),
        this_step_probe=c["step_probe"], this_step_obj=c["step_obj"],
        this_step_pos_correction=c["step_pos"], this_step_tilts=0, masks=None,
        pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]), recon_type="far_field",
        Cs=f(0), defocus_array=np.array([0.0], dtype=f), alpha_near_field=f(0),
        damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(c["rolloff"]),
        propmethod="multislice", this_chopped_sequence=c["sequence"], load_one_by_one=False,
        data_multiplier=f(1), data_pad=0, phase_plate_in_h5=None,
        this_loss_weight=c["loss_weight"], data_bin=1, data_shift_vector=[0, 0],
        upsample_pattern=1, static_background=None, this_step_static_background=0,
        tilt_mode=0, aberration_marker=None, probe_marker=None, aberrations_array=None,
        compute_batch=c["batch"], phase_only_obj=False, beam_current=None,
        this_beam_current_step=0, this_step_aberrations_array=0, default_float=f,
        default_complex=cx, xp=np, is_first_epoch=True, scan_size=None, scan_step_A=1,
        fast_axis_reg_weight_positions=0, slow_axis_reg_weight_positions=0,
        slow_axis_reg_weight_tilts=0, current_deformation_reg_weight_positions=0,
        current_deformation_reg_weight_tilts=0, fast_axis_reg_weight_tilts=0,
        aperture_mask=None, probe_reg_weight=0, current_window_weight=0, current_window=None,
        phase_norm_weight=0, abs_norm_weight=0, atv_weight=0, atv_q=1, atv_p=2,
        mixed_variance_weight=0, mixed_variance_sigma=0.5, wedge_mu=0, beta_wedge=0,
        probe_mod_reg_weight=0, probe_mod_tol=0.05, smart_memory=False, print_flag=0,
        data_simulation_flag=False, data_simulation_exitwave=False, use_padded_intensity=True)
    loss, sse, og, pg, posg = res[0], res[1], res[2], res[3], res[4]
    return loss, sse, og, pg, posg


def build_case(name, seed, W, ny, nx, Z, Mo, Mp, n_scan, step_px, jitter_px, algorithm,
               batch, px=0.2, kV=200.0, alpha=25.0, defocus=80.0, distance=2.0,
               edge_mult=1.0, cutoff=2 / 3, rolloff=0.0, loss_weight=1, step_probe=1,
               step_obj=1, step_pos=0, dose=1e4, double=False, sequence=None,
               integer_positions=False, distances=None):
    rng = np.random.default_rng(seed)
    # inputs are always built in single precision; the double-precision cases upcast the
    # very same inputs so that complex64 and complex128 results are comparable
    cx = np.complex64
    f = np.float32
    truth = synth.gaussian_phase_object(ny, nx, Z, 12 * Z + 20, 0.35, px, 0.2, 0.9, rng,
                                        n_modes=Mo, dtype=cx)
    probe_true = synth.make_probe(W, px, kV, alpha, defocus, Mp,
                                  [0.6, 0.3, 0.1, 0.05, 0.03][:Mp], dose, dtype=cx)
    pos = synth.raster_positions(n_scan, n_scan, step_px, jitter_px, rng)
    if integer_positions:
        pos = np.round(pos)
    ipos, corr = synth.split_positions(pos, int_dtype=np.int32, float_dtype=f)
    assert ipos.max() + W <= min(ny, nx), "object too small for the scan"
    lam = synth.wavelength_A(kV)
    N = ipos.shape[0]
    seq = np.arange(N) if sequence is None else np.asarray(sequence)
    # measured: oracle forward at the truth, plus Poisson noise
    sim = orc.loss_and_direction(truth, probe_true, ipos, corr,
                                 distance if distances is None else np.asarray(distances, f), edge_mult, None,
                                 algorithm, lam, 1, 1, 0, px, px, cutoff, rolloff,
                                 np.arange(N), 1, 64, float_dtype=f, complex_dtype=cx,
                                 simulate=True)
    measured = synth.poisson_patterns(sim, 1.0, rng).astype(f)
    # evaluation point: half the true phase, probe with a small extra defocus
    obj0 = np.exp(0.5j * np.angle(truth)).astype(cx)
    probe0 = synth.make_probe(W, px, kV, alpha, defocus + 15.0, Mp,
                              [0.5, 0.3, 0.2, 0.1, 0.1][:Mp], dose, dtype=cx)
    if double:
        measured = measured.astype(np.float64)
        corr = corr.astype(np.float64)
        obj0 = obj0.astype(np.complex128)
        probe0 = probe0.astype(np.complex128)
    return dict(name=name, double=double, positions=ipos, pos_correction=corr,
                distance=distance, edge_mult=edge_mult, measured=measured,
                algorithm=algorithm, wavelength=lam, step_probe=step_probe,
                step_obj=step_obj, step_pos=step_pos, px=px, cutoff=cutoff,
                rolloff=rolloff, sequence=seq, loss_weight=loss_weight, batch=batch,
                obj=obj0, probe=probe0, distances=None if distances is None else np.asarray(distances, f))


CASES = [
    # the full single-slice benchmark shape: 128^2 object, W=64, 16x16 scan at 2.5 px
    dict(name="single_slice_c64", seed=1, W=64, ny=128, nx=128, Z=1, Mo=1, Mp=1, n_scan=16,
         step_px=2.5, jitter_px=0.0, algorithm="lsq_sqrt", batch=256, px=0.2,
         defocus=100.0, step_pos=1),
    dict(name="single_slice_c128", seed=1, W=64, ny=128, nx=128, Z=1, Mo=1, Mp=1, n_scan=16,
         step_px=2.5, jitter_px=0.0, algorithm="lsq_sqrt", batch=256, px=0.2,
         defocus=100.0, step_pos=1, double=True),
    # multislice, 2 probe modes, Poisson loss, batch remainder (36 = 16 + 16 + 4)
    dict(name="multislice_ml_c64", seed=2, W=64, ny=112, nx=112, Z=4, Mo=1, Mp=2, n_scan=6,
         step_px=6.0, jitter_px=1.5, algorithm="ml", batch=16, px=0.1, kV=300.0,
         alpha=30.0, defocus=40.0, distance=2.0, step_pos=1, dose=1e5),
    dict(name="multislice_ml_c128", seed=2, W=64, ny=112, nx=112, Z=4, Mo=1, Mp=2, n_scan=6,
         step_px=6.0, jitter_px=1.5, algorithm="ml", batch=16, px=0.1, kV=300.0,
         alpha=30.0, defocus=40.0, distance=2.0, step_pos=1, dose=1e5, double=True),
    # object modes, loss weight, squared loss, a non-contiguous sequence
    dict(name="modes_lsq_c64", seed=3, W=64, ny=96, nx=96, Z=2, Mo=2, Mp=2, n_scan=4,
         step_px=7.0, jitter_px=1.0, algorithm="lsq", batch=5, px=0.15, loss_weight=0.7,
         step_pos=1, dose=1e3, sequence=[0, 2, 3, 5, 6, 7, 9, 10, 12, 15]),
    # integer positions (no probe shift), smooth roll-off, thick edge slice
    dict(name="sqrt2_edge_c64", seed=4, W=64, ny=96, nx=96, Z=3, Mo=1, Mp=1, n_scan=4,
         step_px=8.0, jitter_px=0.0, algorithm="lsq_sqrt_2", batch=16, px=0.2,
         edge_mult=1.5, rolloff=0.1, integer_positions=True, dose=1e4),
    # 128-px window, three probe modes, amplitude loss, no position gradient
    dict(name="w128_modes_c64", seed=5, W=128, ny=176, nx=176, Z=3, Mo=1, Mp=3, n_scan=3,
         step_px=12.0, jitter_px=2.0, algorithm="lsq_sqrt", batch=4, px=0.1, kV=300.0,
         alpha=30.0, defocus=50.0, dose=1e5),
    # one distance per slice step (this_distances with Z - 1 entries, multislice_core.py:69-74,
    # 164-174), with a thick first slice; 64 and 128 px windows, and an FP64 twin
    dict(name="distances_ml_c64", seed=6, W=64, ny=112, nx=112, Z=4, Mo=1, Mp=2, n_scan=6,
         step_px=6.0, jitter_px=1.5, algorithm="ml", batch=16, px=0.1, kV=300.0,
         alpha=30.0, defocus=40.0, step_pos=1, dose=1e5, edge_mult=1.3, distances=[1.5, 2.5, 4.0]),
    dict(name="distances_ml_c128", seed=6, W=64, ny=112, nx=112, Z=4, Mo=1, Mp=2, n_scan=6,
         step_px=6.0, jitter_px=1.5, algorithm="ml", batch=16, px=0.1, kV=300.0,
         alpha=30.0, defocus=40.0, step_pos=1, dose=1e5, edge_mult=1.3, distances=[1.5, 2.5, 4.0],
         double=True),
    dict(name="w128_distances_c64", seed=7, W=128, ny=176, nx=176, Z=3, Mo=1, Mp=3, n_scan=3,
         step_px=12.0, jitter_px=2.0, algorithm="lsq_sqrt", batch=4, px=0.1, kV=300.0,
         alpha=30.0, defocus=50.0, dose=1e5, distances=[1.0, 3.0]),
]


def make_loss_cases(pypty, names=None):
    for spec in CASES:
        spec = dict(spec)
        name = spec.pop("name")
        if names and name not in names:
            continue
        c = build_case(name, **spec)
        loss, sse, og, pg, posg = ref_loss_and_direction(pypty, c, c["obj"], c["probe"])
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(
            out, obj=c["obj"], probe=c["probe"], positions=c["positions"],
            pos_correction=c["pos_correction"], measured=c["measured"],
            sequence=c["sequence"],
            scalars=np.array([c["distance"], c["edge_mult"], c["wavelength"], c["px"],
                              c["cutoff"], c["rolloff"], c["loss_weight"], c["batch"],
                              c["step_probe"], c["step_obj"], c["step_pos"]],
                             dtype=np.float64),
            algorithm=np.array(c["algorithm"]), double=np.array(c["double"]),
            ref_loss=np.array(loss, dtype=np.float64), ref_sse=np.array(sse, dtype=np.float64),
            ref_object_grad=og, ref_probe_grad=np.asarray(pg), ref_pos_grad=posg,
            **({} if c["distances"] is None else {"distances": c["distances"]}))
        print("%-20s loss=%.8e sse=%.6e |og|=%.4e -> %s" % (
            name, float(loss), float(sse), np.linalg.norm(og), out))


def make_core_case(pypty):
    """multislice / multislice_grads / scatteradd called directly on small arrays."""
    rng = np.random.default_rng(11)
    B, W, Z, Mp, Mo = 3, 64, 3, 2, 2
    cx = np.complex64
    q2, qx, qy, mask_s, mask = orc.spatial_frequencies(0.2, 0.2, W, 2 / 3, 0, np.float32)
    lam = np.float32(synth.wavelength_A(200.0))
    prop = orc.propagator(np.float32(1.5), lam, q2, qx, qy, mask, cx)[None, :, :, None, None]
    probe_b = (rng.normal(size=(B, W, W, Mp)) + 1j * rng.normal(size=(B, W, W, Mp))).astype(cx)
    obj_b = np.exp(1j * rng.uniform(0, 1, (B, W, W, Z, Mo))).astype(cx)
    g_out = (rng.normal(size=(B, W, W, Mp, Mo)) + 1j * rng.normal(size=(B, W, W, Mp, Mo))).astype(cx)
    stack = np.zeros((B, W, W, Z, Mp, Mo, 1), dtype=cx)
    exit_w = np.zeros((B, W, W, Mp, Mo), dtype=cx)
    m = pypty.multislice_core
    stack, exit_w = m.multislice(probe_b.copy(), obj_b.copy(), Z, Mo, Mp,
                                 np.array([1.5], np.float32), 1.3, lam, q2[None], qx[None],
                                 qy[None], mask_s[None], True, 0, 0, 2 / 3, 0, prop, None,
                                 mask[None], stack, exit_w, 0, 0, np.float32, cx)
    stack_fwd = stack.copy()
    ny = nx = 100
    pos = rng.integers(0, ny - W, (B, 2))
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    my = pos[:, 0][:, None, None] + runy[None]
    mx = pos[:, 1][:, None, None] + runx[None]
    og = np.zeros((ny, nx, Z, Mo), dtype=cx)
    og, pgrad, _ = m.multislice_grads(g_out.copy(), stack, obj_b.copy(), og, None, True,
                                      np.array([1.5], np.float32), 1.3, mask_s[None], lam,
                                      q2[None], qx[None], 0, qy[None], 0, Z, Mo, 0, prop, 0,
                                      2 / 3, 0, 0, B, mask[None], 1, 1, 0, my, mx,
                                      np.float32, cx, True)
    out = os.path.join(HERE, "core_multislice_c64.npz")
    np.savez_compressed(out, probe_b=probe_b, obj_b=obj_b, g_out=g_out, prop=prop[0, :, :, 0, 0],
                        mask=mask, edge_mult=np.array(1.3), positions=pos,
                        ref_stack=stack_fwd[..., 0], ref_exit=exit_w, ref_object_grad=og,
                        ref_probe_grad=pgrad)
    print("core case -> %s" % out)


if __name__ == "__main__":
    pypty = import_reference()
    names = sys.argv[1:]
    make_loss_cases(pypty, names)
    if not names:
        make_core_case(pypty)
