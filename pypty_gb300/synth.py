"""Seeded synthetic specimens, probes and scans for the ptychography workloads.

No public dataset is named for this path, so every workload is built from seeded random
numbers with the shapes and value distributions of the benchmark configurations:

* single-slice: 128x128 px object at 0.2 A/px, 60 Gaussian atoms (sigma 0.4 A, peak phase
  U(0.5, 2) rad), 64 px probe at 200 kV / 25 mrad / 100 A defocus, 16x16 scan at 0.5 A.
* multislice: 512x512 px x 20 slices at 0.1 A/px (2 A apart), 150 atoms per slice
  (sigma 0.3 A, phase U(0.2, 1) rad), 128 px probe at 300 kV / 30 mrad with three
  incoherent modes of power 0.6/0.3/0.1, 32x32 scan at 0.4 A with U(+-0.2 A) jitter.

Physical conventions follow the reference: the electron wavelength formula of
``pypty/utils.py:1721``; positions are in pixels, split into an integer part and a
sub-pixel correction as ``prepare_main_loop_params`` does (``pypty/utils.py:1742-1746``);
the object array layout is ``[y, x, slice, mode]`` and the probe ``[y, x, mode]``.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


def wavelength_A(acc_voltage_kV: float) -> float:
    """Relativistic electron wavelength in Angstrom (``pypty/utils.py:1721``)."""
    return 12.398 / math.sqrt((2 * 511.0 + acc_voltage_kV) * acc_voltage_kV)


def gaussian_phase_object(ny, nx, n_slices, n_atoms, sigma_A, px_A, phase_lo, phase_hi,
                          rng, n_modes=1, dtype=np.complex64):
    """Pure-phase object exp(i*V): V is a sum of isotropic Gaussians per slice.

    Returns an array of shape (ny, nx, n_slices, n_modes). Every object mode holds the
    same slices (incoherent object modes start identical, as a flat start does).
    """
    yy, xx = np.meshgrid(np.arange(ny, dtype=np.float64), np.arange(nx, dtype=np.float64),
                         indexing="ij")
    sig = sigma_A / px_A
    out = np.empty((ny, nx, n_slices, n_modes), dtype=dtype)
    for z in range(n_slices):
        v = np.zeros((ny, nx), dtype=np.float64)
        cy = rng.uniform(0, ny, n_atoms)
        cx = rng.uniform(0, nx, n_atoms)
        amp = rng.uniform(phase_lo, phase_hi, n_atoms)
        r = int(math.ceil(5 * sig))
        for a in range(n_atoms):
            y0, x0 = int(cy[a]), int(cx[a])
            ys = slice(max(0, y0 - r), min(ny, y0 + r + 1))
            xs = slice(max(0, x0 - r), min(nx, x0 + r + 1))
            d2 = (yy[ys, xs] - cy[a]) ** 2 + (xx[ys, xs] - cx[a]) ** 2
            v[ys, xs] += amp[a] * np.exp(-0.5 * d2 / sig ** 2)
        out[:, :, z, :] = np.exp(1j * v)[:, :, None]
    return out


def make_probe(W, px_A, acc_voltage_kV, alpha_mrad, defocus_A, n_modes=1,
               mode_powers=None, dose=1.0, dtype=np.complex64):
    """Defocused aperture probe with ``n_modes`` orthogonal incoherent modes.

    Mode 0 is the aperture-limited defocused probe. Higher modes multiply the aperture
    function by low-order polynomials of (kx, ky) and are Gram-Schmidt orthogonalised. Every
    mode is centred in the window (pixel (W/2, W/2)), as the reference builds its probe
    (``fftshift(ifft2(...))``, ``pypty/utils.py:804``), so that a window at scan position p
    illuminates the object around p + W/2.
    The modes are scaled so that mode j carries ``mode_powers[j]`` of the power and the
    mean far-field pattern of the unshifted probe through vacuum integrates to ``dose``:
    the FFT is unnormalised and modes are averaged, so W^2 * sum_j sum|P_j|^2 / n_modes
    equals ``dose``.
    """
    lam = wavelength_A(acc_voltage_kV)
    f = np.fft.fftfreq(W, px_A)
    kx, ky = np.meshgrid(f, f, indexing="xy")
    k2 = kx ** 2 + ky ** 2
    kmax = alpha_mrad * 1e-3 / lam
    aperture = (k2 <= kmax ** 2).astype(np.float64)
    chi = math.pi * lam * defocus_A * k2
    base = aperture * np.exp(-1j * chi)
    polys = [np.ones_like(kx), kx / kmax, ky / kmax, (kx ** 2 - ky ** 2) / kmax ** 2,
             kx * ky / kmax ** 2, (k2 / kmax ** 2) - 0.5, kx * k2 / kmax ** 3,
             ky * k2 / kmax ** 3]
    if n_modes > len(polys):
        raise ValueError("at most %d probe modes" % len(polys))
    modes = []
    for j in range(n_modes):
        m = np.fft.fftshift(np.fft.ifft2(base * polys[j]))
        for q in modes:
            m = m - np.vdot(q, m) * q
        m = m / np.sqrt(np.vdot(m, m).real)
        modes.append(m)
    if mode_powers is None:
        mode_powers = np.ones(n_modes) / n_modes
    mode_powers = np.asarray(mode_powers, dtype=np.float64)
    mode_powers = mode_powers / mode_powers.sum()
    # W^2 * sum_j |P_j|^2 / n_modes = dose  ->  sum_j |P_j|^2 = dose * n_modes / W^2
    total = dose * n_modes / W ** 2
    probe = np.stack([modes[j] * np.sqrt(total * mode_powers[j]) for j in range(n_modes)],
                     axis=-1)
    return probe.astype(dtype)


def raster_positions(n_y, n_x, step_px, jitter_px=0.0, rng=None, offset_px=0.0):
    """Row-major raster scan (slow axis y) in pixels, optionally jittered uniformly."""
    yy, xx = np.meshgrid(np.arange(n_y) * step_px, np.arange(n_x) * step_px, indexing="ij")
    pos = np.stack([yy.ravel(), xx.ravel()], axis=1).astype(np.float64) + offset_px
    if jitter_px:
        pos = pos + rng.uniform(-jitter_px, jitter_px, pos.shape)
    return pos


def split_positions(pos_px, int_dtype=np.int32, float_dtype=np.float32):
    """Integer + sub-pixel split of pixel positions (``pypty/utils.py:1742-1746``).

    Positions are first shifted so that the smallest is zero, as the reference does
    when it prepares the main loop (``pypty/utils.py:1733-1737``).
    """
    pos = np.array(pos_px, dtype=np.float64)
    pos[:, 0] -= pos[:, 0].min()
    pos[:, 1] -= pos[:, 1].min()
    ipos = np.round(pos).astype(np.int64)
    corr = (pos - ipos).astype(float_dtype)
    return ipos.astype(int_dtype), corr


@dataclasses.dataclass
class Workload:
    """Everything one loss-and-gradient call needs, in the reference's array layouts."""
    name: str
    obj: np.ndarray            # (Ny, Nx, Z, Mo) complex
    probe: np.ndarray          # (W, W, Mp) complex
    positions: np.ndarray      # (N, 2) int [y, x]
    pos_correction: np.ndarray  # (N, 2) float sub-pixel [dy, dx]
    measured: np.ndarray | None  # (N, W, W) float32 detector-plane intensities
    wavelength: float
    pixel_size: float
    slice_distance: float
    algorithm: str
    compute_batch: int
    dose: float
    obj_truth: np.ndarray | None = None


def single_slice_workload(seed=0, dtype=np.complex64):
    """128x128 single-slice object, 64 px probe, 16x16 scan at 2.5 px (amplitude loss)."""
    rng = np.random.default_rng(seed)
    px = 0.2
    W = 64
    truth = gaussian_phase_object(128, 128, 1, 60, 0.4, px, 0.5, 2.0, rng, dtype=dtype)
    probe = make_probe(W, px, 200.0, 25.0, 100.0, 1, None, 1e4, dtype=dtype)
    pos = raster_positions(16, 16, 0.5 / px)
    ipos, corr = split_positions(pos)
    return Workload("single-slice W64 Z1 M1 16x16", truth, probe, ipos, corr, None,
                    wavelength_A(200.0), px, 1.0, "lsq_sqrt", 256, 1e4, truth)


def multislice_workload(seed=0, n_scan=32, dtype=np.complex64, compute_batch=256):
    """512x512x20 object, 128 px probe with 3 modes, 32x32 jittered scan (Poisson loss)."""
    rng = np.random.default_rng(seed)
    px = 0.1
    W = 128
    truth = gaussian_phase_object(512, 512, 20, 150, 0.3, px, 0.2, 1.0, rng, dtype=dtype)
    probe = make_probe(W, px, 300.0, 30.0, 50.0, 3, [0.6, 0.3, 0.1], 1e5, dtype=dtype)
    pos = raster_positions(n_scan, n_scan, 0.4 / px, 0.2 / px, rng)
    ipos, corr = split_positions(pos)
    return Workload("multislice W128 Z20 Mp3 %dx%d" % (n_scan, n_scan), truth, probe, ipos,
                    corr, None, wavelength_A(300.0), px, 2.0, "ml", compute_batch, 1e5,
                    truth)


def poisson_patterns(intensity, dose_scale=1.0, rng=None):
    """Poisson counts of the given expected intensities (float32)."""
    lam = np.clip(intensity * dose_scale, 0, None)
    return rng.poisson(lam).astype(np.float32)
