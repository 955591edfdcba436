"""Golden vectors for the near-field, compressed-detector, beam-current, aberration, tilt,
measured-data preprocessing, detector-upsampling and static-background branches, produced by
running the reference's own NumPy path.

Run where the reference sources are mounted (``PYPTY_REFERENCE_ROOT`` names the
reference checkout; it is required)::

    python tests/golden/make_golden_variants.py [case names]   # every case without names

Every case builds seeded inputs (``pypty_gb300.synth``), simulates measurements with the
variants oracle at the true specimen (patterns plus Poisson noise, or detector coefficients
plus Gaussian noise for the compressed losses), evaluates the reference's
``pypty.objective.loss_and_direction`` (``pypty/objective.py:47``) at a perturbed
object/probe and writes inputs and outputs to ``tests/golden/variant_<case>.npz``.
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
from oracle import variants_oracle as vor  # noqa: E402


def ref_call(pypty, c):
    """The reference with every argument spelled out (signature objective.py:47)."""
    f, cx = (np.float64, np.complex128) if c["double"] else (np.float32, np.complex64)
    if c["tilts"] is not None:
        tilts = c["tilts"].astype(f)
    else:
        tilts = np.zeros((1, 6), dtype=f)
        tilts[0, 2], tilts[0, 3] = c["tan_y"], c["tan_x"]
    masks = None if c["masks"] is None else c["masks"].astype(f)
    bc = None if c["beam_current"] is None else c["beam_current"].astype(f)
    ab = None if c["aberrations"] is None else c["aberrations"].astype(f)
    res = pypty.objective.loss_and_direction(
        this_obj=c["obj"].astype(cx), full_probe=c["probe"].astype(cx),
        this_pos_array=c["positions"].copy(), this_pos_correction=c["pos_correction"].astype(f),
        this_tilt_array=tilts, this_tilts_correction=np.zeros_like(tilts),
        this_distances=(np.array([c["distance"]], dtype=f) if c["distances"] is None
                        else np.asarray(c["distances"], dtype=f)),
        edge_slice_thickness_multiplier=c["edge_mult"],
        measured_array=c["measured"], algorithm_type=c["algorithm"], this_wavelength=f(c["wavelength"]),
        this_step_probe=c["step_probe"], this_step_obj=c["step_obj"], this_step_pos_correction=c["step_pos"],
        this_step_tilts=c["step_tilts"], masks=masks, pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]),
        recon_type=c["recon_type"], Cs=f(c["cs"]),
        defocus_array=(np.array([c["defocus"]], dtype=f) if c["defocus_array"] is None
                       else np.asarray(c["defocus_array"], dtype=f)),
        alpha_near_field=f(c["alpha"]), damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(c["rolloff"]),
        propmethod="multislice", this_chopped_sequence=c["sequence"], load_one_by_one=False,
        data_multiplier=f(c["mult"]), data_pad=c["data_pad"], phase_plate_in_h5=None, this_loss_weight=c["loss_weight"],
        data_bin=1, data_shift_vector=[c["shift0"], c["shift1"]], upsample_pattern=c["upsample"],
        static_background=None if c["static_background"] is None else c["static_background"].astype(f),
        this_step_static_background=c["step_sb"],
        tilt_mode=c["tilt_mode"], aberration_marker=c["aberration_marker"], probe_marker=c["probe_marker"],
        aberrations_array=ab,
        compute_batch=c["batch"], phase_only_obj=False, beam_current=bc,
        this_beam_current_step=c["step_bc"], this_step_aberrations_array=c["step_ab"], default_float=f,
        default_complex=cx, xp=np, is_first_epoch=True, scan_size=None, scan_step_A=1,
        fast_axis_reg_weight_positions=0, slow_axis_reg_weight_positions=0, slow_axis_reg_weight_tilts=0,
        current_deformation_reg_weight_positions=0, current_deformation_reg_weight_tilts=0,
        fast_axis_reg_weight_tilts=0, aperture_mask=None, probe_reg_weight=0, current_window_weight=0,
        current_window=None, phase_norm_weight=0, abs_norm_weight=0, atv_weight=0, atv_q=1, atv_p=2,
        mixed_variance_weight=0, mixed_variance_sigma=0.5, wedge_mu=0, beta_wedge=0, probe_mod_reg_weight=0,
        probe_mod_tol=0.05, smart_memory=False, print_flag=0, data_simulation_flag=False,
        data_simulation_exitwave=False, use_padded_intensity=bool(c["use_padded"]))
    # outer return order (objective.py:967): aberrations gradient before beam-current gradient
    return res[0], res[1], res[2], res[3], res[4], res[8], res[7], res[5], res[6]


def detector_masks(W, n, rng):
    """Segmented annular virtual detectors in detector (fftshifted) order, float32."""
    y, x = np.mgrid[:W, :W] - W // 2
    r = np.hypot(y, x)
    th = np.arctan2(y, x)
    out = []
    for i in range(n):
        r0, r1 = (i // 2) * W / (2 * n) * 1.5, (i // 2 + 1) * W / (2 * n) * 1.5 + 2
        half = (th >= 0) if i % 2 == 0 else (th < 0)
        out.append(((r >= r0) & (r < r1) & half).astype(np.float32) * rng.uniform(0.5, 1.0))
    return np.array(out, dtype=np.float32)


def build_case(name, seed, W, ny, nx, Z, Mp, n_scan, step_px, jitter_px, algorithm, batch, px=0.2, kV=200.0,
               alpha=25.0, probe_defocus=80.0, distance=2.0, edge_mult=1.0, cutoff=2 / 3, rolloff=0.0,
               loss_weight=1.0, step_probe=1, step_obj=1, step_pos=0, dose=1e4, double=False, recon_type="far_field",
               defocus=0.0, cs=0.0, alpha_nf=0.0, tan_x=0.0, tan_y=0.0, n_masks=0, beam_current=False, step_bc=0,
               n_ab_sets=0, n_abs=0, step_ab=0, integer_positions=False, data_pad=0, use_padded=1, shift=(0, 0),
               mult=1.0, tilt_mode=0, tilt_rows=0, tilt_scale=5e-4, step_tilts=0, upsample=1, static=0.0,
               step_sb=0, distances=None, defocus_rows=False, scenarios=0):
    rng = np.random.default_rng(seed)
    cx, f = np.complex64, np.float32
    truth = synth.gaussian_phase_object(ny, nx, Z, 12 * Z + 20, 0.35, px, 0.2, 0.9, rng, dtype=cx)
    probe_true = synth.make_probe(W, px, kV, alpha, probe_defocus, Mp, [0.6, 0.3, 0.1][:Mp], dose, dtype=cx)
    pmarker = None
    if scenarios:   # one probe per scenario (defocus steps of 20 A), positions assigned round robin
        probe_true = np.stack([synth.make_probe(W, px, kV, alpha, probe_defocus + 20.0 * k, Mp,
                                                [0.6, 0.3, 0.1][:Mp], dose, dtype=cx) for k in range(scenarios)], -1)
    pos = synth.raster_positions(n_scan, n_scan, step_px, jitter_px, rng)
    if integer_positions:
        pos = np.round(pos)
    ipos, corr = synth.split_positions(pos, int_dtype=np.int32, float_dtype=f)
    assert ipos.max() + W <= min(ny, nx), "object too small for the scan"
    lam = synth.wavelength_A(kV)
    N = ipos.shape[0]
    if scenarios:
        pmarker = (np.arange(N) % scenarios).astype(np.int64)
    masks = detector_masks(W, n_masks, rng) if n_masks else None
    bc = (1.0 + 0.1 * rng.normal(size=N)).astype(f) if beam_current else None
    ab = (rng.normal(size=(n_ab_sets, n_abs)) * 20.0).astype(f) if n_ab_sets else None
    marker = (np.arange(N) % n_ab_sets).astype(np.int64) if n_ab_sets else None
    # tilt rows [tan_y, tan_x] before / inside / after: one row, or one per position
    tilts = (rng.normal(size=(N if tilt_rows == "per_position" else 1, 6)) * tilt_scale).astype(f) \
        if tilt_rows else None
    # a smooth static background, a fraction `static` of the mean pattern's amplitude
    sb = None
    if static:
        yy, xx = np.mgrid[:W, :W] - W / 2
        sb = (static * np.sqrt(dose / (W * W)) * (0.5 + np.exp(-(yy ** 2 + xx ** 2) / (0.1 * W * W)))
              * rng.uniform(0.8, 1.2, size=(W, W))).astype(f)
    # one near-field defocus per position around the nominal one
    dfa = (defocus + 15.0 * rng.normal(size=N)).astype(f) if defocus_rows else None
    kw = dict(recon_type=recon_type, defocus=defocus if dfa is None else dfa, cs=cs, alpha_near_field=alpha_nf, tan_x=tan_x, tan_y=tan_y,
              masks=masks, beam_current=bc, aberrations=ab, aberration_marker=marker, data_pad=data_pad,
              use_padded_intensity=use_padded, tilts=tilts, tilt_mode=tilt_mode, upsample_pattern=upsample,
              static_background=sb, probe_marker=pmarker)
    dist = distance if distances is None else np.asarray(distances, f)
    sim = vor.loss_and_direction_variants(truth, probe_true, ipos, corr, dist, edge_mult, None, algorithm, lam,
                                          1, 1, 0, px, px, cutoff, rolloff, np.arange(N), 1, 64, simulate=True, **kw)
    if n_masks:
        measured = (sim * (1.0 + 0.02 * rng.normal(size=sim.shape))).astype(f)
    else:
        measured = synth.poisson_patterns(sim, 1.0, rng).astype(f)
        # stored so that the reference's per-batch shift and multiplier (objective.py:411)
        # bring it back near the model
        measured = (np.roll(measured, (-shift[0], -shift[1]), axis=(1, 2)) / mult).astype(f)
    obj0 = np.exp(0.5j * np.angle(truth)).astype(cx)
    probe0 = synth.make_probe(W, px, kV, alpha, probe_defocus + 15.0, Mp, [0.5, 0.3, 0.2][:Mp], dose, dtype=cx)
    if scenarios:
        probe0 = np.stack([synth.make_probe(W, px, kV, alpha, probe_defocus + 15.0 + 20.0 * k, Mp,
                                            [0.5, 0.3, 0.2][:Mp], dose, dtype=cx) for k in range(scenarios)], -1)
    if double:
        measured, corr = measured.astype(np.float64), corr.astype(np.float64)
        obj0, probe0 = obj0.astype(np.complex128), probe0.astype(np.complex128)
    return dict(name=name, double=double, positions=ipos, pos_correction=corr, distance=distance,
                edge_mult=edge_mult, measured=measured, algorithm=algorithm, wavelength=lam, step_probe=step_probe,
                step_obj=step_obj, step_pos=step_pos, px=px, cutoff=cutoff, rolloff=rolloff,
                sequence=np.arange(N), loss_weight=loss_weight, batch=batch, obj=obj0, probe=probe0,
                recon_type=recon_type, defocus=defocus, cs=cs, alpha=alpha_nf, tan_x=tan_x, tan_y=tan_y, masks=masks,
                beam_current=bc, step_bc=step_bc, aberrations=ab, aberration_marker=marker, step_ab=step_ab,
                data_pad=data_pad, use_padded=use_padded, shift0=shift[0], shift1=shift[1], mult=mult,
                tilts=tilts, tilt_mode=tilt_mode, step_tilts=step_tilts, upsample=upsample,
                static_background=None if sb is None else (sb.astype(np.float64) if double else sb),
                step_sb=step_sb, distances=None if distances is None else np.asarray(distances, f),
                defocus_array=dfa, probe_marker=pmarker)


BASE = dict(W=64, ny=112, nx=112, Z=2, Mp=2, n_scan=5, step_px=8.0, jitter_px=1.2, batch=10, px=0.15, kV=300.0,
            alpha=30.0, probe_defocus=40.0, dose=1e5)
CASES = [
    # near field: CTF with defocus, Cs and an inside tilt; position gradient
    dict(BASE, name="near_c64", seed=31, algorithm="lsq_sqrt", recon_type="near_field", defocus=60.0, cs=2e5,
         tan_x=2e-3, tan_y=-1e-3, step_pos=1),
    dict(BASE, name="near_c128", seed=31, algorithm="lsq_sqrt", recon_type="near_field", defocus=60.0, cs=2e5,
         tan_x=2e-3, tan_y=-1e-3, step_pos=1, double=True),
    # near field, Poisson loss, integer positions, thick first slice
    dict(BASE, name="near_ml_c64", seed=32, algorithm="ml", recon_type="near_field", defocus=80.0, Z=3,
         edge_mult=1.4, integer_positions=True),
    # compressed detectors (far field, inside tilt)
    dict(BASE, name="lsq_compressed_c64", seed=33, algorithm="lsq_compressed", n_masks=6, tan_x=1e-3, step_pos=1),
    dict(BASE, name="gauss_compressed_c64", seed=34, algorithm="gauss_compressed", n_masks=6),
    dict(BASE, name="poisson_compressed_c64", seed=35, algorithm="poisson_compressed", n_masks=6, loss_weight=0.5),
    # beam current and aberration plates, integer positions (the plates act in the forward model)
    dict(BASE, name="current_aberr_c64", seed=36, algorithm="ml", beam_current=True, step_bc=1, n_ab_sets=3,
         n_abs=7, step_ab=1, integer_positions=True),
    dict(BASE, name="current_aberr_c128", seed=36, algorithm="ml", beam_current=True, step_bc=1, n_ab_sets=3,
         n_abs=7, step_ab=1, integer_positions=True, double=True),
    # measured detector smaller than the window: zero-padded measurements, or the cropped model
    # pattern (objective.py:411, 516-517, 592-593)
    dict(BASE, name="pad_c64", seed=38, algorithm="ml", data_pad=6, step_pos=1),
    dict(BASE, name="crop_c64", seed=39, algorithm="lsq_sqrt", data_pad=6, use_padded=0),
    # the per-batch shift vector and multiplier of the measured patterns (utils.py:626-647)
    dict(BASE, name="shift_mult_c64", seed=40, algorithm="lsq", shift=(2, -3), mult=1.5, Mp=1),
    # beam tilts (objective.py:302-345, 464-499, 605-673; multislice_core.py:76-77, 178-182):
    # per-position inside tilts with their gradient
    dict(BASE, name="tilt0_rows_c64", seed=41, algorithm="ml", tilt_mode=0, tilt_rows="per_position",
         step_tilts=1),
    # one inside tilt row: batches of one position (the reference raises for more)
    dict(BASE, name="tilt0_single_c64", seed=42, algorithm="lsq_sqrt", tilt_mode=0, tilt_rows="single",
         step_tilts=1, batch=1, n_scan=3),
    # after the specimen, per position; one slice (the exit wave is band-limited first)
    dict(BASE, name="tilt1_rows_z1_c64", seed=43, algorithm="lsq_sqrt", tilt_mode=1, tilt_rows="per_position",
         step_tilts=1, Z=1),
    # before the specimen, one row, one probe mode (the reference's x grid quirk), shifts; the
    # amplitude loss (a Poisson loss on one coherent mode divides by near-zero intensities at the
    # pattern's dark pixels, where any two FP32 evaluations differ)
    dict(BASE, name="tilt2_single_c64", seed=44, algorithm="lsq_sqrt", tilt_mode=2, tilt_rows="single",
         step_tilts=1, Mp=1, step_pos=1),
    # inside and after, near field, per position
    dict(BASE, name="tilt3_near_rows_c64", seed=45, algorithm="lsq_sqrt", tilt_mode=3, tilt_rows="per_position",
         step_tilts=1, recon_type="near_field", defocus=60.0, cs=2e5),
    # before, inside and after, per position, with shifts, and its FP64 twin
    dict(BASE, name="tilt4_rows_c64", seed=46, algorithm="ml", tilt_mode=4, tilt_rows="per_position", step_tilts=1,
         step_pos=1),
    dict(BASE, name="tilt4_rows_c128", seed=46, algorithm="ml", tilt_mode=4, tilt_rows="per_position",
         step_tilts=1, step_pos=1, double=True),
    # the same with sub-pixel shifts: the shift spectrum excludes the plates (objective.py:461, 471)
    dict(BASE, name="current_aberr_shift_c64", seed=37, algorithm="lsq_sqrt", beam_current=True, step_bc=1,
         n_ab_sets=2, n_abs=4, step_ab=1, step_pos=1),
    # detector upsampling (objective.py:523-524, 590-591): 2 x 2 block sums of the model
    # pattern; alone, with the cropped pattern, and with zero-padded measurements
    dict(BASE, name="upsample2_c64", seed=47, algorithm="ml", upsample=2, step_pos=1),
    dict(BASE, name="upsample2_crop_c64", seed=48, algorithm="lsq_sqrt", upsample=2, data_pad=6, use_padded=0),
    dict(BASE, name="upsample2_pad_c64", seed=49, algorithm="ml", upsample=2, data_pad=6, use_padded=1,
         shift=(1, -2)),
    # static background with its gradient (objective.py:359-361, 525-526, 588-589): far field,
    # near field, a compressed loss, and an FP64 twin
    dict(BASE, name="static_c64", seed=50, algorithm="lsq_sqrt", static=0.3, step_sb=1, step_pos=1),
    dict(BASE, name="static_c128", seed=50, algorithm="lsq_sqrt", static=0.3, step_sb=1, step_pos=1, double=True),
    dict(BASE, name="static_near_c64", seed=51, algorithm="ml", static=0.2, step_sb=1, recon_type="near_field",
         defocus=60.0, cs=2e5),
    dict(BASE, name="static_compressed_c64", seed=52, algorithm="lsq_compressed", n_masks=6, static=0.2,
         step_sb=1),
    # one distance per slice step (multislice_core.py:69-74, 164-182): per-position inside tilts
    # with their gradient and a thick first slice; tilts after the specimen, per position (each
    # step's propagator then takes the position's own inside tilt); near field
    dict(BASE, name="distances_tilt0_rows_c64", seed=53, algorithm="ml", Z=3, tilt_mode=0,
         tilt_rows="per_position", step_tilts=1, edge_mult=1.2, distances=[1.5, 2.5], step_pos=1),
    dict(BASE, name="distances_tilt1_rows_c64", seed=54, algorithm="lsq_sqrt", Z=3, tilt_mode=1,
         tilt_rows="per_position", step_tilts=1, distances=[1.0, 3.0]),
    dict(BASE, name="distances_near_c64", seed=55, algorithm="lsq_sqrt", Z=3, recon_type="near_field",
         defocus=60.0, cs=2e5, tan_x=2e-3, distances=[1.2, 2.2], step_pos=1),
    # near field with one defocus per position (objective.py:413-418): batches of one position,
    # the only size for which the reference's (B,) defocus broadcasts; with an inside tilt, and
    # with per-position inside tilts and their gradient
    dict(BASE, name="near_defocus_rows_c64", seed=56, algorithm="lsq_sqrt", recon_type="near_field", defocus=60.0,
         cs=2e5, tan_x=2e-3, defocus_rows=True, batch=1, n_scan=4, step_pos=1),
    dict(BASE, name="near_defocus_tilt0_c64", seed=57, algorithm="ml", recon_type="near_field", defocus=50.0,
         cs=1e5, defocus_rows=True, batch=1, n_scan=4, tilt_mode=0, tilt_rows="per_position", step_tilts=1),
    # several probe scenarios (a 4D probe with probe_marker, objective.py:355-356, 443-444,
    # 700-701): sub-pixel shifts with the position gradient, and its FP64 twin; with beam
    # current and aberration plates; with a tilt before the specimen
    dict(BASE, name="scenarios_c64", seed=58, algorithm="ml", scenarios=3, step_pos=1),
    dict(BASE, name="scenarios_c128", seed=58, algorithm="ml", scenarios=3, step_pos=1, double=True),
    dict(BASE, name="scenarios_current_aberr_c64", seed=59, algorithm="lsq_sqrt", scenarios=2, beam_current=True,
         step_bc=1, n_ab_sets=2, n_abs=4, step_ab=1, step_pos=1),
    dict(BASE, name="scenarios_tilt4_c64", seed=60, algorithm="lsq_sqrt", scenarios=2, tilt_mode=4,
         tilt_rows="per_position", step_tilts=1, step_pos=1),
]


def main(names=None):
    pypty = import_reference()
    for spec in CASES:
        spec = dict(spec)
        name = spec.pop("name")
        if names and name not in names:
            continue
        c = build_case(name, **spec)
        loss, sse, og, pg, posg, bcg, abg, tg, sbg = ref_call(pypty, c)
        out = os.path.join(HERE, "variant_" + name + ".npz")
        none = np.zeros(0, np.float32)
        np.savez_compressed(
            out, obj=c["obj"], probe=c["probe"], positions=c["positions"], pos_correction=c["pos_correction"],
            measured=c["measured"], sequence=c["sequence"],
            scalars=np.array([c["distance"], c["edge_mult"], c["wavelength"], c["px"], c["cutoff"], c["rolloff"],
                              c["loss_weight"], c["batch"], c["step_probe"], c["step_obj"], c["step_pos"],
                              c["defocus"], c["cs"], c["alpha"], c["tan_x"], c["tan_y"], c["step_bc"], c["step_ab"],
                              c["data_pad"], c["use_padded"], c["shift0"], c["shift1"], c["mult"], c["tilt_mode"],
                              c["step_tilts"], c["upsample"], c["step_sb"]],
                             dtype=np.float64),
            algorithm=np.array(c["algorithm"]), recon_type=np.array(c["recon_type"]), double=np.array(c["double"]),
            masks=none if c["masks"] is None else c["masks"],
            beam_current=none if c["beam_current"] is None else c["beam_current"],
            aberrations=none if c["aberrations"] is None else c["aberrations"],
            aberration_marker=np.zeros(0, np.int64) if c["aberration_marker"] is None else c["aberration_marker"],
            ref_loss=np.array(loss, dtype=np.float64), ref_sse=np.array(sse, dtype=np.float64),
            ref_object_grad=og, ref_probe_grad=np.asarray(pg), ref_pos_grad=posg,
            ref_beam_current_grad=np.asarray(bcg), ref_aberrations_grad=np.asarray(abg),
            tilts=none if c["tilts"] is None else c["tilts"], ref_tilts_grad=np.asarray(tg),
            static_background=none if c["static_background"] is None else c["static_background"],
            ref_static_grad=np.asarray(sbg), distances=none if c["distances"] is None else c["distances"],
            defocus_array=none if c["defocus_array"] is None else c["defocus_array"],
            probe_marker=np.zeros(0, np.int64) if c["probe_marker"] is None else c["probe_marker"])
        print("%-26s loss=%.8e sse=%.6e |og|=%.4e |bcg|=%.3e |abg|=%.3e -> %s" % (
            name, float(loss), float(sse), np.linalg.norm(og), np.linalg.norm(np.asarray(bcg)),
            np.linalg.norm(np.asarray(abg)), os.path.basename(out)))


if __name__ == "__main__":
    main(sys.argv[1:])
