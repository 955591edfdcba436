"""NumPy restatement of pypty's far-field multislice loss-and-gradient path.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): this module checks the CUDA path; it
is never part of it.

Supported flag set (the one the GPU path implements): far-field propagation,
``propmethod="multislice"``, no beam tilts (tilt_mode 0, tilts zero), no phase plates,
aberration arrays, beam-current fluctuations, static background, data padding, binning or
compressed detectors, one slice distance or one per slice step (``distance`` an array with
more than one entry, ``multislice_core.py:69-74, 164-174``), algorithms ``lsq_sqrt``, ``ml``, ``lsq``
and ``lsq_sqrt_2``, sub-pixel probe shifts and the position gradient. Regularisers are off.

Every step cites the reference line it restates. The arithmetic is done in the array dtype
the caller passes (complex64 for parity with the GPU path, complex128 for the FP64 oracle),
with ``scipy.fft`` (pocketfft) as the reference's CPU path uses (``pypty/fft.py:4-6``).
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft

PI_TRUNC = 3.141592654      # literal used by the reference propagators (multislice_core.py:72)
TWO_PI_TRUNC = 6.2831855    # literal used by the reference shift ramps (objective.py:309)


# --------------------------------------------------------------------------- fft wrappers
def fft2(a, axes=(0, 1)):
    """``pypty/fft.py:114-134``: unnormalised 2D DFT."""
    return sfft.fft2(a, axes=axes)


def ifft2(a, axes=(0, 1)):
    """``pypty/fft.py:136-156``: 2D inverse DFT scaled by 1/(n0*n1)."""
    return sfft.ifft2(a, axes=axes)


def shift_fft2(a, axes=(0, 1)):
    """``pypty/fft.py:91-112``: fftshift(fft2(a))."""
    return sfft.fftshift(sfft.fft2(a, axes=axes), axes=axes)


def ifft2_ishift(a, axes=(0, 1)):
    """``pypty/fft.py:158-178``: ifft2(ifftshift(a))."""
    return sfft.ifft2(sfft.ifftshift(a, axes=axes), axes=axes)


# --------------------------------------------------------------------------- frequencies
def spatial_frequencies(px, py, W, damping_cutoff, smooth_rolloff, float_dtype):
    """``pypty/utils.py:153-199`` ``create_spatial_frequencies``.

    Returns q2, qx, qy, exclude_mask (fftshifted) and exclude_mask_ishift, each (W, W).
    """
    qx, qy = np.meshgrid(sfft.fftfreq(W, px), sfft.fftfreq(W, py), indexing="xy")
    qx, qy = qx.astype(float_dtype), qy.astype(float_dtype)
    q2 = qx ** 2 + qy ** 2
    if damping_cutoff is None:
        damping_cutoff = 2
    if damping_cutoff < 0:
        damping_cutoff = 2 / 3
    max_x = np.max(qx)
    r_max = (max_x * damping_cutoff) ** 2
    mask = (q2 <= r_max).astype(float_dtype)
    if smooth_rolloff != 0:
        r0 = (max_x * (damping_cutoff - smooth_rolloff)) ** 2
        sel = q2 > r0
        mask[sel] *= (0.5 * (1 + np.cos(PI_TRUNC * (q2 - r0) / (r_max - r0))))[sel]
    mask = mask.astype(float_dtype)
    return q2, qx, qy, sfft.fftshift(mask), mask


def propagator(distance, wavelength, q2, qx, qy, mask, complex_dtype, tan_x=0.0, tan_y=0.0):
    """Fresnel propagator of one slice step, ``pypty/objective.py:337-345``."""
    p = np.exp(-PI_TRUNC * 1j * distance * (wavelength * q2 + 2 * (qx * tan_x + qy * tan_y)))
    return (p * mask).astype(complex_dtype)


def shift_ramp_tables(W, mask, complex_dtype):
    """Sub-pixel shift exponents, ``pypty/objective.py:308-313``.

    Returns (smy, smx), each (W, W) complex: -2*pi*i*f * mask with the truncated 2*pi.
    """
    fx, fy = np.meshgrid(sfft.fftfreq(W), sfft.fftfreq(W), indexing="xy")
    smx = (-TWO_PI_TRUNC * 1j * fx).astype(complex_dtype) * mask
    smy = (-TWO_PI_TRUNC * 1j * fy).astype(complex_dtype) * mask
    return smy.astype(complex_dtype), smx.astype(complex_dtype)


# --------------------------------------------------------------------------- multislice
def multislice(probe_b, obj_b, prop, edge_mult):
    """Forward split-step multislice, ``pypty/multislice_core.py:61-82``.

    probe_b: (B, W, W, Mp); obj_b: (B, W, W, Z, Mo); prop: (W, W) propagator (mask applied),
    or a list of one per slice step (per-slice distances, ``multislice_core.py:69-71``).
    Returns the conjugated input-wave stack (B, W, W, Z, Mp, Mo) and the exit wave
    (B, W, W, Mp, Mo).
    """
    B, W, _, Z, Mo = obj_b.shape
    Mp = probe_b.shape[-1]
    stack = np.empty((B, W, W, Z, Mp, Mo), dtype=obj_b.dtype)
    wave = np.repeat(probe_b[:, :, :, :, None], Mo, axis=-1)
    for z in range(Z):
        stack[:, :, :, z] = wave
        wave = wave * obj_b[:, :, :, z:z + 1, :]
        if z < Z - 1:
            p = prop[z] if isinstance(prop, list) else prop
            if edge_mult > 1 and z == 0:
                p = p ** edge_mult
            wave = fft2(wave, axes=(1, 2))
            wave = wave * p[None, :, :, None, None]
            wave = ifft2(wave, axes=(1, 2))
    return np.conjugate(stack), wave


def multislice_grads(g, stack_conj, obj_b, prop, edge_mult, mask):
    """Adjoint multislice, ``pypty/multislice_core.py:158-200``.

    g: dL/d(exit wave) (B, W, W, Mp, Mo). Returns the band-limited per-position object
    gradient windows (B, W, W, Z, Mo) and the probe gradient (B, W, W, Mp).
    """
    Z = obj_b.shape[3]
    obj_c = np.conjugate(obj_b)
    contrib = np.empty_like(stack_conj)
    for z in range(Z - 1, -1, -1):
        contrib[:, :, :, z] = stack_conj[:, :, :, z] * g
        g = g * obj_c[:, :, :, z:z + 1, :]
        if z > 0:
            # the step from slice z - 1 (multislice_core.py:164-172: P(-d) = conj P(d))
            p = np.conjugate(prop[z - 1] if isinstance(prop, list) else prop)
            if edge_mult > 1 and z == 1:
                p = p ** edge_mult
            g = fft2(g, axes=(1, 2))
            g = g * p[None, :, :, None, None]
            g = ifft2(g, axes=(1, 2))
    grad = contrib.sum(axis=4)                          # sum over probe modes (:188)
    grad = fft2(grad, axes=(1, 2))
    grad = grad * mask[None, :, :, None, None]
    grad = ifft2(grad, axes=(1, 2))
    probe_grad = g.sum(axis=-1)                         # sum over object modes (:197)
    return grad, probe_grad


def scatteradd(full, masky, maskx, chop):
    """``pypty/multislice_core.py:206-230``: unbuffered in-order add (``np.add.at``)."""
    np.add.at(full, (masky, maskx), chop)


# --------------------------------------------------------------------------- loss
def loss_terms(pattern, measured, algorithm):
    """Loss, sse and dL/dI for one batch, ``pypty/objective.py:527-558``.

    Returns (loss_sum, sse_sum, dLdI). The sums are accumulated in the array dtype, as the
    reference does with ``cp.sum``.
    """
    if algorithm == "lsq_sqrt":
        sse = np.sum((measured - pattern) ** 2)
        ps = np.sqrt(pattern)
        ms = np.sqrt(measured)
        d = ps - ms
        loss = np.sum(d ** 2)
        ps[ps == 0] = 1
        return loss, sse, d / ps
    if algorithm == "ml":
        d = pattern - measured
        sse = np.sum(d ** 2)
        zero = pattern == 0
        loss = np.sum(pattern - measured * np.log(pattern + zero))
        pattern = pattern.copy()
        pattern[zero] = 1
        return loss, sse, d / pattern
    if algorithm == "lsq":
        t = np.sum((pattern - measured) ** 2)
        return t, t, 2 * (pattern - measured)
    if algorithm == "lsq_sqrt_2":
        t = (measured - pattern) ** 2
        sse = np.sum(t)
        nz = measured > 0.5
        loss = 0.5 * np.sum(t[nz] / measured[nz]) + np.sum(pattern[~nz])
        d = np.ones_like(pattern)
        d[nz] = pattern[nz] / measured[nz] - 1
        return loss, sse, d
    raise ValueError("unsupported algorithm %r" % algorithm)


# --------------------------------------------------------------------------- full path
def loss_and_direction(obj, probe, positions, pos_correction, distance, edge_mult, measured,
                       algorithm, wavelength, step_probe, step_obj, step_pos, pixel_size_x,
                       pixel_size_y, damping_cutoff, smooth_rolloff, sequence, loss_weight,
                       compute_batch, float_dtype=np.float32, complex_dtype=np.complex64,
                       simulate=False):
    """Restatement of ``pypty/objective.py:47-967`` for the supported flag set.

    obj (Ny, Nx, Z, Mo); probe (W, W, Mp); positions (N, 2) int [y, x]; pos_correction
    (N, 2) float; measured (N, W, W) float (indexed by ``sequence``). Returns
    (loss, sse, object_grad, probe_grad, pos_grad). With ``simulate=True`` it returns the
    simulated mean-over-modes patterns (len(sequence), W, W) instead (the
    ``data_simulation_flag`` path, ``objective.py:524-526``).
    """
    obj = np.asarray(obj, dtype=complex_dtype)
    probe = np.asarray(probe, dtype=complex_dtype)
    W = probe.shape[0]
    Mp = probe.shape[2]
    Z, Mo = obj.shape[2], obj.shape[3]
    coherent = Mp == 1 and Mo == 1
    # the reference receives these as default_float scalars (pypty/iterative.py:111-112,139)
    pixel_size_x, pixel_size_y = float_dtype(pixel_size_x), float_dtype(pixel_size_y)
    damping_cutoff, smooth_rolloff = float_dtype(damping_cutoff), float_dtype(smooth_rolloff)
    q2, qx, qy, mask_s, mask = spatial_frequencies(pixel_size_x, pixel_size_y, W,
                                                   damping_cutoff, smooth_rolloff, float_dtype)
    smy, smx = shift_ramp_tables(W, mask, complex_dtype)
    dists = np.asarray(distance, dtype=float_dtype).reshape(-1)
    if dists.shape[0] > 1:   # one propagator per slice step (is_single_dist false)
        prop = [propagator(dists[z], float_dtype(wavelength), q2, qx, qy, mask, complex_dtype)
                for z in range(Z - 1)]
    else:
        prop = propagator(dists[0], float_dtype(wavelength), q2, qx, qy, mask, complex_dtype)
    probe_shift = bool(np.sum(pos_correction.astype(np.float64) ** 2) != 0.0) or bool(step_pos)
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    object_grad = np.zeros_like(obj)
    probe_grad = np.zeros((W, W, Mp), dtype=complex_dtype)
    pos_grad = np.zeros_like(pos_correction)
    loss, sse = 0, 0
    probe_f = fft2(probe) if probe_shift else None     # objective.py:471
    sim = []
    seq = np.asarray(sequence)
    for i in range(0, len(seq), compute_batch):
        tcs = seq[i:i + compute_batch]
        meas = None if measured is None else np.array(measured[tcs])
        ys = positions[tcs, 0][:, None, None]
        xs = positions[tcs, 1][:, None, None]
        my, mx = ys + runy[None], xs + runx[None]
        # window gather + band limit, objective.py:436-441
        ob = obj[my, mx, :, :]
        ob = ifft2(fft2(ob, axes=(1, 2)) * mask[None, :, :, None, None], axes=(1, 2))
        ob = ob.astype(complex_dtype)
        # sub-pixel probe shift, objective.py:469-476
        if probe_shift:
            corr = pos_correction[tcs]
            ramp = np.exp(smx[None] * corr[:, 1:2, None] + smy[None] * corr[:, 0:1, None])
            ramp = ramp * mask[None]
            pb = ifft2(probe_f[None] * ramp[:, :, :, None], axes=(1, 2))
        else:
            pb = np.repeat(probe[None], len(tcs), axis=0)
        pb = pb.astype(complex_dtype)
        stack, exit_wave = multislice(pb, ob, prop, edge_mult)
        # far field, objective.py:501-512
        wave = shift_fft2(exit_wave, axes=(1, 2)) * mask_s[None, :, :, None, None]
        pattern = np.abs(wave) ** 2
        pattern = pattern[:, :, :, 0, 0] if coherent else np.mean(pattern, (-1, -2))
        if simulate:
            sim.append(pattern)
            continue
        l_b, s_b, dldi = loss_terms(pattern, meas, algorithm)
        loss = loss + l_b
        sse = sse + s_b
        if not coherent:
            dldi = dldi / (Mp * Mo)                     # objective.py:586-587
        # far-field adjoint, objective.py:595-597
        dwave = dldi[:, :, :, None, None] * wave * (loss_weight * W * W)
        g = ifft2_ishift(dwave, axes=(1, 2))
        g = g.astype(complex_dtype)
        grad_w, pgrad = multislice_grads(g, stack, ob, prop, edge_mult, mask)
        if step_obj:
            scatteradd(object_grad, my, mx, grad_w.astype(complex_dtype))
        # probe-shift adjoint and position gradient, objective.py:641-658
        if probe_shift:
            fpg = fft2(pgrad, axes=(1, 2)) * np.conjugate(ramp)[:, :, :, None]
            pgrad = ifft2(fpg, axes=(1, 2))
            if step_pos:
                smg = np.conjugate(probe_f)[None] * fpg
                sh = -2 / (W * W)
                gy = sh * np.sum(np.real(smy[None, :, :, None] * smg), (1, 2, 3))
                gx = sh * np.sum(np.real(smx[None, :, :, None] * smg), (1, 2, 3))
                pos_grad[tcs, 0] = gy
                pos_grad[tcs, 1] = gx
        if step_probe:
            probe_grad = probe_grad + np.sum(pgrad, 0)  # objective.py:703
    if simulate:
        return np.concatenate(sim, 0)
    loss = loss * loss_weight                            # objective.py:742
    if loss != loss:
        raise ValueError('A very specific bad thing. Loss is Nan.')
    if step_probe:                                      # objective.py:927-933
        probe_grad = ifft2(fft2(probe_grad) * mask[:, :, None])
    return loss, sse, object_grad, probe_grad.astype(complex_dtype), pos_grad
