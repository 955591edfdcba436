"""NumPy restatement of the other propagation / loss / probe branches of pypty's
``objective.loss_and_direction``: near-field propagation, compressed-detector losses,
beam-current fluctuations, per-position aberration phase plates, beam tilts and the
per-batch measured-data preprocessing.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): this module checks the CUDA path; it
is never part of it.

Flag set (beyond ``ptycho_oracle``'s): the per-batch measured-data preprocessing of
``objective.py:411-412`` (shift vector, multiplier, zero padding by ``data_pad`` with
``use_padded_intensity``, or the cropped model pattern without it, ``objective.py:516-517,
592-593``); ``recon_type`` "far_field" or "near_field" with one
defocus or one per position (``is_single_defocus`` false, ``objective.py:413-418``) and
spherical aberration ``Cs`` (``objective.py:504-508,
598-604``); algorithms
``lsq_compressed``, ``gauss_compressed`` and ``poisson_compressed`` with detector masks
(``objective.py:560-585``); ``beam_current`` with its gradient (``objective.py:448-452,
687-697``); ``aberrations_array`` / ``aberration_marker`` with their gradient
(``objective.py:324-329, 459-463, 676-684``); beam tilts (``tilt_mode`` 0-4, one tilt row or
one per position, with the tilt gradient: ``objective.py:302-345, 464-499, 605-673``,
``multislice_core.py:76-77, 178-182``); the detector upsampling (``upsample_pattern``,
``objective.py:523-524, 590-591``) and a 2D static background with its gradient
(``objective.py:359-361, 525-526, 588-589``). Every step cites the reference line it restates;
dtypes follow the reference in single or double precision.

The near-field partial-coherence correction (``alpha_near_field > 0``) is not restated: the
reference's envelope has shape (1, 1, W, W) (``objective.py:514``, ``q2`` already carries a
leading axis), its forward transforms the wrong axes and its adjoint raises a broadcasting
error (``objective.py:600`` into ``multislice_core.py:161``), so the branch has no reference
result to match; this function raises ValueError for it, as the reference raises.

Reference behaviours restated as they are: with a probe shift active, the forward probe is
built from the spectrum taken before the aberration plate (``objective.py:461, 471-476``:
``this_probe_fourier`` is not updated by the plate or a tilt after it) while the adjoint
still applies their conjugates; with one probe mode the before-tilt gradient's x component
uses the x grid's first column (``objective.py:664``); one tilt row with inside-tilt
refinement raises for batches of more than one position (``multislice_core.py:181``).
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft

from .ptycho_oracle import (fft2, ifft2, ifft2_ishift, loss_terms, multislice, multislice_grads, propagator,
                            scatteradd, shift_fft2, shift_ramp_tables, spatial_frequencies)

COMPRESSED = ("lsq_compressed", "gauss_compressed", "poisson_compressed")


def convert_num_to_nmab(num_abs):
    """Krivanek (n, m, a/b) order of the first ``num_abs`` aberrations, ``utils.py:1272-1308``."""
    max_n = int(np.ceil(0.5 * (-5 + np.sqrt(25 + 8 * num_abs))))
    ns, ms, abs_ = [], [], []
    # numpy int64 orders, as the reference's np.arange loops: they promote the float32
    # frequency arrays of ctf_matrix to float64 (k_r ** n, m * phi)
    for n in np.arange(1, max_n + 1, 1):
        for m in np.arange((n + 1) % 2, n + 2, 2):
            if m == 0:
                ns.append(n), ms.append(m), abs_.append("")
            else:
                ns.append(n), ms.append(m), abs_.append("a")
                ns.append(n), ms.append(m), abs_.append("b")
    return ns[:num_abs], ms[:num_abs], abs_[:num_abs]


def ctf_matrix(kx, ky, num_abs, wavelength):
    """``utils.py:1333-1368`` ``get_ctf_matrix``: (num_abs, W, W) float64 phase basis."""
    ns, ms, abs_ = convert_num_to_nmab(num_abs)
    k_r = np.sqrt(kx ** 2 + ky ** 2)
    phi = np.angle(kx + 1j * ky)
    A = np.zeros((num_abs,) + k_r.shape)
    for i in range(num_abs):
        term = (k_r ** (ns[i] + 1)) / (ns[i] + 1)
        if abs_[i] == "a":
            term = term * np.cos(ms[i] * phi)
        elif abs_[i] == "b":
            term = term * np.sin(ms[i] * phi)
        A[i] = term
    A *= 6.283185307179586 / wavelength
    return A


def aberration_polynomials(qx, qy, num_abs, wavelength, complex_dtype):
    """``objective.py:326-327``: -1j * get_ctf_matrix(lambda qx, lambda qy) in the complex dtype."""
    return (-1j * ctf_matrix(wavelength * qx, wavelength * qy, num_abs, wavelength)).astype(complex_dtype)


def compressed_terms(pattern, measured, masks, algorithm):
    """Loss, sse and dL/dI of the compressed-detector algorithms, ``objective.py:560-585``.

    pattern (B, W, W); measured (B, n_masks); masks (n_masks, W, W)."""
    coeffs = np.sum(pattern[:, None, :, :] * masks[None, :, :, :], axis=(2, 3))
    if algorithm == "lsq_compressed":
        diff = coeffs - measured
        t = np.sum(diff ** 2)
        diff = diff * 2
        return t, t, np.sum(masks[None] * diff[:, :, None, None], axis=1)
    if algorithm == "gauss_compressed":
        ms = np.sqrt(measured)
        cs = np.sqrt(coeffs)
        sse = np.sum((coeffs - measured) ** 2)
        d = cs - ms
        loss = np.sum(d ** 2)
        cs[cs == 0] = 1
        d = d / cs
        return loss, sse, np.sum(masks[None] * d[:, :, None, None], axis=1)
    if algorithm == "poisson_compressed":
        d = coeffs - measured
        sse = np.sum(d ** 2)
        coeffs = coeffs.copy()
        coeffs[coeffs == 0] = 1
        loss = np.sum(coeffs - measured * np.log(coeffs))
        d = d / coeffs
        return loss, sse, np.sum(masks[None] * d[:, :, None, None], axis=1)
    raise ValueError("unsupported compressed algorithm %r" % algorithm)


def preprocess_measured(dataset, data_shift_vector, data_multiplier, data_pad):
    """``utils.py:626-652`` ``preprocess_dataset`` as ``objective.py:411-412`` calls it per
    batch (not compressed, ``force_pad``, no binning): roll by the shift vector and zero the
    rows / columns the reference zeroes, scale, zero-pad."""
    s0, s1 = int(data_shift_vector[0]), int(data_shift_vector[1])
    if s0 != 0:
        dataset = np.roll(dataset, s0, axis=1)
        if s0 > 0:
            dataset[:, -s0:, :] = 0
        else:
            dataset[:, :-s0, :] = 0
    if s1 != 0:
        dataset = np.roll(dataset, s1, axis=2)
        if s1 > 0:
            dataset[:, :, -s1:] = 0
        else:
            dataset[:, :, :-s1] = 0
    if data_multiplier != 1:
        dataset = dataset * data_multiplier
    return np.pad(dataset, [[0, 0], [data_pad, data_pad], [data_pad, data_pad]])


def downsample_pattern(pattern, up):
    """``utils.py:403-426`` ``downsample_something_3d``: sums over up x up blocks (both axes
    cut to a multiple of up of axis 1's length, as the reference does)."""
    n = pattern.shape[1]
    k = n // up
    p = pattern[:, :up * k, :up * k]
    return p.reshape(pattern.shape[0], k, up, k, up).sum(axis=(2, 4))


def tilt_grids(W, pixel_size_x, pixel_size_y, wavelength, complex_dtype):
    """Real-space tilt ramps of ``objective.py:303-307``: (y_grid, x_grid), each (W, W)
    purely imaginary, 2*pi*i*W*px/lambda times the fftshifted frequencies (complex128, then the
    complex dtype)."""
    fx, fy = np.meshgrid(sfft.fftshift(sfft.fftfreq(W)), sfft.fftshift(sfft.fftfreq(W)), indexing="xy")
    xg = (fx * 6.2831855j * W * pixel_size_x / wavelength).astype(complex_dtype)
    yg = (fy * 6.2831855j * W * pixel_size_y / wavelength).astype(complex_dtype)
    return yg, xg


def loss_and_direction_variants(obj, probe, positions, pos_correction, distance, edge_mult, measured, algorithm,
                                wavelength, step_probe, step_obj, step_pos, pixel_size_x, pixel_size_y,
                                damping_cutoff, smooth_rolloff, sequence, loss_weight, compute_batch,
                                recon_type="far_field", defocus=0.0, cs=0.0, alpha_near_field=0.0, tan_x=0.0,
                                tan_y=0.0, masks=None, beam_current=None, step_beam_current=0, aberrations=None,
                                aberration_marker=None, step_aberrations=0, data_pad=0, use_padded_intensity=True,
                                data_shift_vector=(0, 0), data_multiplier=1.0, tilts=None, tilt_mode=0,
                                step_tilts=0, upsample_pattern=1, static_background=None,
                                step_static_background=0, probe_marker=None, float_dtype=np.float32,
                                complex_dtype=np.complex64, simulate=False):
    """Restatement of ``pypty/objective.py:47-967`` for the flag set in the module docstring.

    tilts: (N_tilts, 6) rows [tan_y, tan_x] before / inside / after the specimen (the
    reference's tilt array plus its correction; one row for all positions or one per position),
    used by ``tilt_mode`` 0-4 (``objective.py:302-345, 464-499``); without it one inside tilt
    (tan_x, tan_y). ``upsample_pattern`` sums the model pattern over blocks before the loss
    (``objective.py:523-524, 590-591``); ``static_background`` (W, W) adds its square, band
    limited, to every pattern (``objective.py:359-361, 525-526``) and
    ``step_static_background`` accumulates its gradient (``objective.py:588-589``). A 4D probe
    (W, W, Mp, S) with ``probe_marker`` (one scenario index per position) gives every position
    its scenario's probe and returns the (W, W, Mp, S) probe gradient (``objective.py:355-356,
    443-444, 700-701, 754-755, 929-931``). Returns
    (loss, sse, object_grad, probe_grad, pos_grad, beam_current_grad, aberrations_grad,
    tilts_grad, static_background_grad); the beam-current, aberration and static-background
    gradients are 0 (zeros for a given background) when the feature is off (the reference's
    zero-initialised accumulators, ``objective.py:377, 381-382``).
    ``simulate=True`` returns the model patterns at the measured detector's shape (cropped by
    ``data_pad``, block-summed by ``upsample_pattern``) or, for compressed algorithms, the
    coefficients (len(sequence), n_masks); ``simulate="exit"`` the exit waves (len(sequence),
    W, W, Mp, Mo) after a tilt after the specimen (``data_simulation_exitwave``).
    """
    f = float_dtype
    obj = np.asarray(obj, dtype=complex_dtype)
    probe = np.asarray(probe, dtype=complex_dtype)
    W, Mp = probe.shape[0], probe.shape[2]
    Z, Mo = obj.shape[2], obj.shape[3]
    coherent = Mp == 1 and Mo == 1
    near = recon_type == "near_field"
    compressed = algorithm in COMPRESSED
    px, py = f(pixel_size_x), f(pixel_size_y)
    lam = f(wavelength)
    q2, qx, qy, mask_s, mask = spatial_frequencies(px, py, W, f(damping_cutoff), f(smooth_rolloff), f)
    smy, smx = shift_ramp_tables(W, mask, complex_dtype)
    if tilts is None:
        tilts = np.zeros((1, 6), dtype=f)
        tilts[0, 2], tilts[0, 3] = tan_y, tan_x
    tilts = np.asarray(tilts, dtype=f)
    single_tilt = tilts.shape[0] == 1
    inside_grad = bool(step_tilts) and tilt_mode in (0, 3, 4)
    before = tilt_mode in (2, 4)
    after = tilt_mode in (1, 3, 4)
    if before or after:
        yg, xg = tilt_grids(W, px, py, lam, complex_dtype)
        yx = np.stack((yg[None, :, :, None], xg[None, :, :, None]), axis=1)   # (1, 2, W, W, 1), objective.py:307
    # one propagator for all positions unless per-position inside tilts (objective.py:330-345)
    same_prop = single_tilt or tilt_mode in (1, 2)
    # per-slice distances (is_single_dist false): multislice builds each step's propagator from
    # the batch's own inside tilts, for every tilt mode (multislice_core.py:69-71, 164-170)
    dists = np.asarray(distance, dtype=f).reshape(-1)
    per_step = dists.shape[0] > 1 and Z > 1
    d = dists[0]
    pos_prop = not same_prop or (per_step and not single_tilt)
    if not pos_prop:
        t0 = tilts[0]
        if per_step:
            prop = [propagator(dists[z], lam, q2, qx, qy, mask, complex_dtype, t0[3], t0[2]) for z in range(Z - 1)]
        else:
            prop = propagator(d, lam, q2, qx, qy, mask, complex_dtype, t0[3], t0[2])
    probe_shift = bool(np.sum(np.asarray(pos_correction, np.float64) ** 2) != 0.0) or bool(step_pos)
    fluct = beam_current is not None
    morph = aberrations is not None
    if fluct:
        beam_current = np.asarray(beam_current, dtype=f)
    if morph:                                                           # objective.py:324-329
        aberrations = np.asarray(aberrations, dtype=f)
        polys = aberration_polynomials(qx, qy, aberrations.shape[1], lam, complex_dtype)
        plates = np.exp(np.sum(polys[None] * aberrations[:, :, None, None], 1)) * mask
    if compressed and data_pad != 0:
        raise ValueError("data_pad with compressed detectors: the masks would need the cropped shape")
    if near:
        # defocus_array with one entry per position (is_single_defocus false): each batch takes
        # its positions' entries (objective.py:413-418); the reference's (B,) array broadcasts
        # against the (1, W, W) grids only for batches of one position
        dfa = np.asarray(defocus, dtype=f).reshape(-1)
        per_pos_defocus = dfa.shape[0] > 1
        dfc = dfa[0]
        if alpha_near_field > 0:
            raise ValueError("near-field alpha_near_field > 0: the reference raises (objective.py:600)")
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    object_grad = np.zeros_like(obj)
    scen = probe_marker is not None and probe.ndim == 4                 # multiple_scenarios, objective.py:285
    if scen:
        probe_s = np.moveaxis(probe, 3, 0)                              # (S, W, W, Mp), objective.py:355-356
        probe_marker = np.asarray(probe_marker)
        probe_grad = np.zeros(probe_s.shape, dtype=complex_dtype)
    else:
        probe_grad = np.zeros((W, W, Mp), dtype=complex_dtype)
    pos_grad = np.zeros_like(pos_correction)
    tilts_grad = np.zeros_like(tilts)
    up = int(upsample_pattern)
    if static_background is not None:                                   # objective.py:359-361, 377
        static_background = np.asarray(static_background, dtype=f)
        static_square = (static_background[None, :, :] ** 2) * mask_s[None]
        sb_grad = np.zeros_like(static_background)
    else:
        sb_grad = 0
    bc_grad = np.zeros_like(beam_current) if fluct else 0
    ab_grad = np.zeros_like(aberrations) if morph else 0
    helper2 = step_probe or step_beam_current or step_aberrations
    helper3 = helper2 or (bool(step_tilts) and before)
    helper4 = helper3 or step_pos
    loss, sse = 0, 0
    sim = []
    seq = np.asarray(sequence)
    for i in range(0, len(seq), compute_batch):
        tcs = seq[i:i + compute_batch]
        B = len(tcs)
        tind = [0] if single_tilt else tcs
        tl = tilts[tind][:, :, None, None]                              # (n, 6, 1, 1)
        ty_b, tx_b, ty_i, tx_i, ty_a, tx_a = np.split(tl, 6, axis=1)    # each (n, 1, 1, 1)
        ty_i, tx_i = ty_i[:, :, :, 0], tx_i[:, :, :, 0]                 # (n, 1, 1)
        my = positions[tcs, 0][:, None, None] + runy[None]
        mx = positions[tcs, 1][:, None, None] + runx[None]
        ob = obj[my, mx, :, :]                                          # objective.py:436-441
        ob = ifft2(fft2(ob, axes=(1, 2)) * mask[None, :, :, None, None], axes=(1, 2)).astype(complex_dtype)
        this_probe = probe_s[probe_marker[tcs]] if scen else probe[None]   # objective.py:443-447
        probe_f = None
        if fluct:                                                       # objective.py:448-452
            bc = np.abs(beam_current[tcs])
            before_fluct = this_probe
            this_probe = this_probe * bc[:, None, None, None]
        if morph:                                                       # objective.py:459-463
            plate = plates[np.asarray(aberration_marker)[tcs]]
            probe_f = fft2(this_probe, axes=(1, 2))
            before_ab = probe_f * 1
            this_probe = ifft2(before_ab * plate[:, :, :, None], axes=(1, 2))
        if before:                                                      # objective.py:464-467
            tmask_b = np.exp(xg[None, :, :, None] * tx_b + yg[None, :, :, None] * ty_b)
            probe_before_tilt = this_probe
            this_probe = probe_before_tilt * tmask_b
        if probe_shift:                                                 # objective.py:470-476
            if probe_f is None:
                probe_f = fft2(this_probe, axes=(1, 2))
            corr = pos_correction[tcs]
            ramp = np.exp(smx[None] * corr[:, 1:2, None] + smy[None] * corr[:, 0:1, None]) * mask[None]
            this_probe = ifft2(probe_f * ramp[:, :, :, None], axes=(1, 2))
        if this_probe.shape[0] == 1 and B > 1:
            this_probe = np.repeat(this_probe, B, axis=0)
        this_probe = this_probe.astype(complex_dtype)
        if not pos_prop:
            prop_b = [p[None] for p in prop] if per_step else prop[None]
        else:                                                           # objective.py:482-484
            def pos_propagator(dz):
                return (np.exp(-3.141592654j * dz * (lam * q2 + 2 * (qx * tx_i + qy * ty_i))) * mask).astype(
                    complex_dtype)
            prop_b = [pos_propagator(dists[z]) for z in range(Z - 1)] if per_step else pos_propagator(d)
        stack, exit_wave, spec_stack = multislice_tilted(this_probe, ob, prop_b, edge_mult, inside_grad)
        if after:                                                       # objective.py:490-499
            tmask_a = np.exp(xg[None, :, :, None] * tx_a + yg[None, :, :, None] * ty_a)[:, :, :, :, None]
            if Z == 1:
                exit_wave = ifft2(fft2(exit_wave, axes=(1, 2)) * mask[None, :, :, None, None], axes=(1, 2))
            exit_before_tilt = exit_wave
            exit_wave = exit_before_tilt * tmask_a
        if simulate == "exit":                                          # objective.py:518-520
            sim.append(exit_wave)
            continue
        if near and per_pos_defocus:
            dfc = dfa[tcs][:, None, None]                               # (B, 1, 1)
        if near:                                                        # objective.py:504-508
            ctf = (np.exp(-3.141592654j * (((lam * q2 + 2 * (qx * tx_i + qy * ty_i)) * dfc)
                                          + (0.5 * f(cs) * lam ** 3 * q2 ** 2))) * mask)[:, :, :, None, None]
            fourier_exit = fft2(exit_wave, axes=(1, 2))
            wave = ifft2(fourier_exit * ctf, axes=(1, 2))
        else:                                                           # objective.py:502-503
            wave = shift_fft2(exit_wave, axes=(1, 2)) * mask_s[None, :, :, None, None]
        pattern = np.abs(wave) ** 2
        pattern = pattern[:, :, :, 0, 0] if coherent else np.mean(pattern, (-1, -2))
        if data_pad != 0 and not use_padded_intensity:                 # objective.py:516-517
            pattern = pattern[:, data_pad:-data_pad, data_pad:-data_pad]
        if up != 1:                                                     # objective.py:523-524
            pattern = downsample_pattern(pattern, up)
        if static_background is not None:                               # objective.py:525-526
            pattern = pattern + static_square
        if simulate:
            if data_pad != 0 and use_padded_intensity:
                po = data_pad // up
                pattern = pattern[:, po:pattern.shape[1] - po, po:pattern.shape[2] - po]
            if compressed:
                sim.append(np.sum(pattern[:, None] * masks[None], axis=(2, 3)))
            else:
                sim.append(pattern)
            continue
        meas = 1 * np.asarray(measured)[tcs]
        if not compressed:                                              # objective.py:411-412
            meas = preprocess_measured(meas, data_shift_vector, data_multiplier,
                                       (data_pad * use_padded_intensity) // up)   # utils.py:649-651
        if compressed:
            l_b, s_b, dldi = compressed_terms(pattern, meas, masks, algorithm)
        else:
            l_b, s_b, dldi = loss_terms(pattern, meas, algorithm)
        loss = loss + l_b
        sse = sse + s_b
        if not coherent:
            dldi = dldi / (Mp * Mo)                                     # objective.py:586-587
        if step_static_background and static_background is not None:    # objective.py:588-589
            sb_grad = sb_grad + np.sum(dldi, 0) * 2 * static_background * loss_weight
        if up != 1:                                                     # objective.py:590-591
            dldi = np.repeat(np.repeat(dldi, up, axis=1), up, axis=2)
        if not use_padded_intensity and data_pad != 0:                  # objective.py:592-593
            dldi = np.pad(dldi, [[0, 0], [data_pad, data_pad], [data_pad, data_pad]])
        if near:                                                        # objective.py:598-619
            dwave = wave * np.expand_dims(dldi, (-1, -2))
            fwg = loss_weight * fft2(dwave, axes=(1, 2)) * np.conjugate(ctf)
            g = ifft2(fwg, axes=(1, 2))
            if inside_grad:
                rsc = -12.566370614359172 / (W * W)
                fwg = fwg * np.conjugate(fourier_exit)
                if coherent:
                    gx = np.sum(np.imag(fwg[:, :, :, 0, 0] * qx * dfc), (1, 2))
                    gy = np.sum(np.imag(fwg[:, :, :, 0, 0] * qy * dfc), (1, 2))
                else:
                    d5 = dfc[:, :, :, None, None] if per_pos_defocus else dfc
                    gx = np.sum(np.imag(fwg * qx[None, :, :, None, None] * d5), (1, 2, 3, 4))
                    gy = np.sum(np.imag(fwg * qy[None, :, :, None, None] * d5), (1, 2, 3, 4))
                if single_tilt:
                    gx, gy = np.sum(gx), np.sum(gy)
                tilts_grad[tind, 2] += gy * rsc
                tilts_grad[tind, 3] += gx * rsc
        else:                                                           # objective.py:595-597
            dwave = dldi[:, :, :, None, None] * wave * (loss_weight * W * W)
            g = ifft2_ishift(dwave, axes=(1, 2))
        if after:                                                       # objective.py:620-639
            g = g * np.conjugate(tmask_a)
            if step_tilts:
                kern = -2 * g * np.conjugate(exit_before_tilt)
                if coherent:
                    dt = np.sum(np.real(kern[:, None, :, :, 0, 0] * yx[:, :, :, :, 0]), (2, 3), dtype=f)
                else:
                    dt = np.sum(np.real(kern[:, None] * yx[:, :, :, :, :, None]), (2, 3, 4, 5), dtype=f)
                if single_tilt:
                    tilts_grad[0, 4:] += np.sum(dt, 0)
                else:
                    tilts_grad[tind, 4:] = dt
            if Z == 1:
                g = ifft2(fft2(g, axes=(1, 2)) * mask[None, :, :, None, None], axes=(1, 2))
        g = g.astype(complex_dtype)
        # a single tilt row with more than one position per batch makes the reference add a
        # (B,) vector into one row of tilts_grad (multislice_core.py:180-182): NumPy raises
        # ValueError there, as the reference does
        grad_w, pgrad = multislice_grads_tilted(g, stack, spec_stack, ob, prop_b, edge_mult, mask,
                                                list(dists[:Z - 1]) if per_step else d, qx, qy,
                                                tilts_grad if inside_grad else None, tind)
        if step_obj:
            scatteradd(object_grad, my, mx, grad_w.astype(complex_dtype))
        if not helper4:
            continue
        fpg = None
        if probe_shift:                                                 # objective.py:643-658
            fpg = fft2(pgrad, axes=(1, 2)) * np.conjugate(ramp)[:, :, :, None]
            pgrad = ifft2(fpg, axes=(1, 2))
            if step_pos:
                smg = np.conjugate(probe_f) * fpg
                sh = -2 / (W * W)
                pos_grad[tcs, 0] = sh * np.sum(np.real(smy[None, :, :, None] * smg), (1, 2, 3))
                pos_grad[tcs, 1] = sh * np.sum(np.real(smx[None, :, :, None] * smg), (1, 2, 3))
        if helper3:
            if before:                                                  # objective.py:660-673
                pgrad = pgrad * np.conjugate(tmask_b)
                if step_tilts:
                    kern = -2 * pgrad * np.conjugate(probe_before_tilt)
                    if Mp == 1:
                        # yx[:, :, :, 0] selects x = 0 (shape (1, 2, W, 1)): the x component uses
                        # the grid's first column for every x, as the reference computes it
                        dt = np.sum(np.real(kern[:, None, :, :, 0] * yx[:, :, :, 0]), (2, 3), dtype=f)
                    else:
                        dt = np.sum(np.real(kern[:, None] * yx), (2, 3, 4), dtype=f)
                    if single_tilt:
                        tilts_grad[0, :2] += np.sum(dt, 0)
                    else:
                        tilts_grad[tind, :2] = dt
            if helper2:
                if morph:                                               # objective.py:676-684
                    fpg = fft2(pgrad, axes=(1, 2))
                    fpg = fpg * np.conjugate(plate[:, :, :, None])
                    pgrad = ifft2(fpg, axes=(1, 2))
                    if step_aberrations:
                        sh = 2 / (W * W)
                        defgr = sh * np.sum(np.real((fpg * np.conjugate(before_ab))[:, None]
                                                    * np.conjugate(polys[None, :, :, :, None])), axis=(2, 3, 4),
                                            dtype=f)
                        np.add.at(ab_grad, np.asarray(aberration_marker)[tcs], defgr)
                if step_probe or step_beam_current:
                    if fluct:                                           # objective.py:687-697
                        if step_beam_current:
                            bc_grad[tcs] = 2 * np.sign(bc) * np.sum(np.real(pgrad * np.conjugate(before_fluct)),
                                                                    (1, 2, 3))
                        if step_probe:
                            pgrad = pgrad * bc[:, None, None, None]
                    if step_probe:
                        if scen:                                        # objective.py:700-701, 972-989
                            np.add.at(probe_grad, probe_marker[tcs], pgrad)
                        else:
                            probe_grad = probe_grad + np.sum(pgrad, 0)  # objective.py:703
    if simulate:
        return np.concatenate(sim, 0)
    loss = loss * loss_weight                                           # objective.py:742
    if loss != loss:
        raise ValueError('A very specific bad thing. Loss is Nan.')
    if step_probe and scen:                                             # objective.py:754-755, 927-933
        probe_grad = np.moveaxis(probe_grad, 0, 3)
        probe_grad = ifft2(fft2(probe_grad) * mask[:, :, None, None])
    elif step_probe:                                                    # objective.py:927-933
        probe_grad = ifft2(fft2(probe_grad) * mask[:, :, None])
    return (loss, sse, object_grad, np.asarray(probe_grad).astype(complex_dtype), pos_grad, bc_grad, ab_grad,
            tilts_grad, sb_grad)


def multislice_tilted(probe_b, obj_b, prop_b, edge_mult, keep_spectra):
    """Forward multislice with one propagator per position (prop_b (n, W, W), n = 1 or B, or
    a list of those per slice step), ``multislice_core.py:61-82``; with ``keep_spectra`` also
    the conjugated spectra
    FFT(psi_z O_z) of every propagated slice (the second stack channel, ``:76-77``)."""
    B, W, _, Z, Mo = obj_b.shape
    Mp = probe_b.shape[-1]
    stack = np.empty((B, W, W, Z, Mp, Mo), dtype=obj_b.dtype)
    spec = np.zeros((B, W, W, Z, Mp, Mo), dtype=obj_b.dtype) if keep_spectra else None
    wave = np.repeat(probe_b[:, :, :, :, None], Mo, axis=-1)
    for z in range(Z):
        stack[:, :, :, z] = wave
        wave = wave * obj_b[:, :, :, z:z + 1, :]
        if z < Z - 1:
            p = prop_b[z] if isinstance(prop_b, list) else prop_b
            if edge_mult > 1 and z == 0:
                p = p ** edge_mult
            wave = fft2(wave, axes=(1, 2))
            if keep_spectra:
                spec[:, :, :, z] = wave
            wave = wave * p[:, :, :, None, None]
            wave = ifft2(wave, axes=(1, 2))
    return np.conjugate(stack), wave, (None if spec is None else np.conjugate(spec))


def multislice_grads_tilted(g, stack_conj, spec_conj, obj_b, prop_b, edge_mult, mask, distance, qx, qy,
                            tilts_grad, tind):
    """Adjoint multislice with per-position propagators, ``multislice_core.py:158-200``; with
    ``tilts_grad`` it adds the inside-tilt gradient terms of every step into rows ``tind``
    (``:178-182``). Returns (gradient windows, probe gradient)."""
    Z = obj_b.shape[3]
    W = obj_b.shape[1]
    obj_c = np.conjugate(obj_b)
    contrib = np.empty_like(stack_conj)
    for z in range(Z - 1, -1, -1):
        contrib[:, :, :, z] = stack_conj[:, :, :, z] * g
        g = g * obj_c[:, :, :, z:z + 1, :]
        if z > 0:
            # the step from slice z - 1 and its distance (multislice_core.py:164-172)
            p = np.conjugate(prop_b[z - 1] if isinstance(prop_b, list) else prop_b)
            dist = 1 * (distance[z - 1] if isinstance(distance, list) else distance)
            if edge_mult > 1 and z == 1:
                p = p ** edge_mult
                dist *= edge_mult
            g = fft2(g, axes=(1, 2))
            g = g * p[:, :, :, None, None]
            if tilts_grad is not None:
                sh = -12.566370614359172 * dist / (W * W)
                dldp = np.sum(spec_conj[:, :, :, z - 1] * g, (3, 4))
                tilts_grad[tind, 3] += sh * np.sum(np.imag(dldp * qx), (1, 2))
                tilts_grad[tind, 2] += sh * np.sum(np.imag(dldp * qy), (1, 2))
            g = ifft2(g, axes=(1, 2))
    grad = contrib.sum(axis=4)
    grad = fft2(grad, axes=(1, 2))
    grad = grad * mask[None, :, :, None, None]
    grad = ifft2(grad, axes=(1, 2))
    probe_grad = g.sum(axis=-1)
    return grad, probe_grad
