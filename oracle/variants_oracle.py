"""NumPy restatement of the other propagation / loss / probe branches of pypty's
``objective.loss_and_direction``: near-field propagation, compressed-detector losses,
beam-current fluctuations, per-position aberration phase plates and a single inside beam
tilt.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): this module checks the CUDA path; it
is never part of it.

Flag set (beyond ``ptycho_oracle``'s): the per-batch measured-data preprocessing of
``objective.py:411-412`` (shift vector, multiplier, zero padding by ``data_pad`` with
``use_padded_intensity``, or the cropped model pattern without it, ``objective.py:516-517,
592-593``); ``recon_type`` "far_field" or "near_field" with one
defocus (``is_single_defocus``) and spherical aberration ``Cs`` (``objective.py:504-508,
598-604``); algorithms
``lsq_compressed``, ``gauss_compressed`` and ``poisson_compressed`` with detector masks
(``objective.py:560-585``); ``beam_current`` with its gradient (``objective.py:448-452,
687-697``); ``aberrations_array`` / ``aberration_marker`` with their gradient
(``objective.py:324-329, 459-463, 676-684``); one inside tilt (``tilt_mode`` 0, a single tilt
row, ``objective.py:337-345, 505``) without tilt gradients. Every step cites the reference
line it restates; dtypes follow the reference in single or double precision.

The near-field partial-coherence correction (``alpha_near_field > 0``) is not restated: the
reference's envelope has shape (1, 1, W, W) (``objective.py:514``, ``q2`` already carries a
leading axis), its forward transforms the wrong axes and its adjoint raises a broadcasting
error (``objective.py:600`` into ``multislice_core.py:161``), so the branch has no reference
result to match; this function raises ValueError for it, as the reference raises.

Two reference behaviours are restated as they are: with a probe shift active, the forward
probe is built from the spectrum taken before the aberration plate (``objective.py:461,
471-476``: ``this_probe_fourier`` is not updated by the plate) while the adjoint still applies
the plate's conjugate; and the gradient arrays come back in the reference's order.
"""
from __future__ import annotations

import numpy as np

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


def loss_and_direction_variants(obj, probe, positions, pos_correction, distance, edge_mult, measured, algorithm,
                                wavelength, step_probe, step_obj, step_pos, pixel_size_x, pixel_size_y,
                                damping_cutoff, smooth_rolloff, sequence, loss_weight, compute_batch,
                                recon_type="far_field", defocus=0.0, cs=0.0, alpha_near_field=0.0, tan_x=0.0,
                                tan_y=0.0, masks=None, beam_current=None, step_beam_current=0, aberrations=None,
                                aberration_marker=None, step_aberrations=0, data_pad=0, use_padded_intensity=True,
                                data_shift_vector=(0, 0), data_multiplier=1.0, float_dtype=np.float32,
                                complex_dtype=np.complex64, simulate=False):
    """Restatement of ``pypty/objective.py:47-967`` for the flag set in the module docstring.

    Returns (loss, sse, object_grad, probe_grad, pos_grad, beam_current_grad,
    aberrations_grad); the last two are 0 when the feature is off (as the reference's
    zero-initialised accumulators, ``objective.py:381-382``). ``simulate=True`` returns the
    model patterns (len(sequence), W, W) or, for compressed algorithms, the coefficients
    (len(sequence), n_masks); with ``data_pad`` the patterns are cropped to the measured
    (W - 2 data_pad)² detector.
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
    # the reference's tilt arrays are (1, 6, 1, 1) default_float rows (objective.py:343, 434-435)
    tx, ty = np.full((1, 1), tan_x, dtype=f), np.full((1, 1), tan_y, dtype=f)
    prop = propagator(f(distance), lam, q2, qx, qy, mask, complex_dtype, tx, ty)
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
    if near:                                                            # objective.py:505, 516
        dfc = f(defocus)
        ctf = (np.exp(-3.141592654j * (((lam * q2 + 2 * (qx * tx + qy * ty)) * dfc)
                                      + (0.5 * f(cs) * lam ** 3 * q2 ** 2))) * mask)[None, :, :, None, None]
        if alpha_near_field > 0:
            raise ValueError("near-field alpha_near_field > 0: the reference raises (objective.py:600)")
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    object_grad = np.zeros_like(obj)
    probe_grad = np.zeros((W, W, Mp), dtype=complex_dtype)
    pos_grad = np.zeros_like(pos_correction)
    bc_grad = np.zeros_like(beam_current) if fluct else 0
    ab_grad = np.zeros_like(aberrations) if morph else 0
    helper2 = step_probe or step_beam_current or step_aberrations
    helper4 = helper2 or step_pos
    loss, sse = 0, 0
    sim = []
    seq = np.asarray(sequence)
    for i in range(0, len(seq), compute_batch):
        tcs = seq[i:i + compute_batch]
        B = len(tcs)
        my = positions[tcs, 0][:, None, None] + runy[None]
        mx = positions[tcs, 1][:, None, None] + runx[None]
        ob = obj[my, mx, :, :]                                          # objective.py:436-441
        ob = ifft2(fft2(ob, axes=(1, 2)) * mask[None, :, :, None, None], axes=(1, 2)).astype(complex_dtype)
        this_probe = probe[None]                                        # objective.py:443-447
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
        if probe_shift:                                                 # objective.py:470-476
            if probe_f is None:
                probe_f = fft2(this_probe, axes=(1, 2))
            corr = pos_correction[tcs]
            ramp = np.exp(smx[None] * corr[:, 1:2, None] + smy[None] * corr[:, 0:1, None]) * mask[None]
            this_probe = ifft2(probe_f * ramp[:, :, :, None], axes=(1, 2))
        if this_probe.shape[0] == 1 and B > 1:
            this_probe = np.repeat(this_probe, B, axis=0)
        this_probe = this_probe.astype(complex_dtype)
        stack, exit_wave = multislice(this_probe, ob, prop, edge_mult)
        if near:                                                        # objective.py:506-508
            wave = ifft2(fft2(exit_wave, axes=(1, 2)) * ctf, axes=(1, 2))
        else:                                                           # objective.py:502-503
            wave = shift_fft2(exit_wave, axes=(1, 2)) * mask_s[None, :, :, None, None]
        pattern = np.abs(wave) ** 2
        pattern = pattern[:, :, :, 0, 0] if coherent else np.mean(pattern, (-1, -2))
        if data_pad != 0 and not use_padded_intensity:                 # objective.py:516-517
            pattern = pattern[:, data_pad:-data_pad, data_pad:-data_pad]
        if simulate:
            if data_pad != 0 and use_padded_intensity:
                pattern = pattern[:, data_pad:-data_pad, data_pad:-data_pad]
            if compressed:
                sim.append(np.sum(pattern[:, None] * masks[None], axis=(2, 3)))
            else:
                sim.append(pattern)
            continue
        meas = 1 * np.asarray(measured)[tcs]
        if not compressed:                                              # objective.py:411-412
            meas = preprocess_measured(meas, data_shift_vector, data_multiplier, data_pad * use_padded_intensity)
        if compressed:
            l_b, s_b, dldi = compressed_terms(pattern, meas, masks, algorithm)
        else:
            l_b, s_b, dldi = loss_terms(pattern, meas, algorithm)
        loss = loss + l_b
        sse = sse + s_b
        if not coherent:
            dldi = dldi / (Mp * Mo)                                     # objective.py:586-587
        if not use_padded_intensity and data_pad != 0:                  # objective.py:592-593
            dldi = np.pad(dldi, [[0, 0], [data_pad, data_pad], [data_pad, data_pad]])
        if near:                                                        # objective.py:598-604
            dwave = wave * np.expand_dims(dldi, (-1, -2))
            fwg = loss_weight * fft2(dwave, axes=(1, 2)) * np.conjugate(ctf)
            g = ifft2(fwg, axes=(1, 2))
        else:                                                           # objective.py:595-597
            dwave = dldi[:, :, :, None, None] * wave * (loss_weight * W * W)
            g = ifft2_ishift(dwave, axes=(1, 2))
        g = g.astype(complex_dtype)
        grad_w, pgrad = multislice_grads(g, stack, ob, prop, edge_mult, mask)
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
        if helper2:
            if morph:                                                   # objective.py:676-684
                if fpg is None:
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
                if fluct:                                               # objective.py:687-697
                    if step_beam_current:
                        bc_grad[tcs] = 2 * np.sign(bc) * np.sum(np.real(pgrad * np.conjugate(before_fluct)),
                                                                (1, 2, 3))
                    if step_probe:
                        pgrad = pgrad * bc[:, None, None, None]
                if step_probe:
                    probe_grad = probe_grad + np.sum(pgrad, 0)          # objective.py:703
    if simulate:
        return np.concatenate(sim, 0)
    loss = loss * loss_weight                                           # objective.py:742
    if loss != loss:
        raise ValueError('A very specific bad thing. Loss is Nan.')
    if step_probe:                                                      # objective.py:927-933
        probe_grad = ifft2(fft2(probe_grad) * mask[:, :, None])
    return (loss, sse, object_grad, np.asarray(probe_grad).astype(complex_dtype), pos_grad, bc_grad, ab_grad)
