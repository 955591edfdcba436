"""NumPy restatement of pypty's optimizer step: ``fourier_clean`` and ``bfgs_update``.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): this module checks the CUDA path;
it is never part of it.

Follows ``pypty/utils.py:102-150`` (``fourier_clean``), ``pypty/utils.py:326-368``
(Wolfe conditions), ``pypty/objective.py:1119-1141`` (``make_states_orthogonal``) and
``pypty/iterative.py:440-1049`` / ``1055-1103`` (``bfgs_update`` /
``reset_bfgs_history``) for the flag set the GPU path supports: object, probe and
position-correction refinement; no phase-only objects, probe Fourier tuning, tilts,
static background, aberrations, beam current, charge flipping, Gaussian filters, object
resizing or position puzzling. Arithmetic in the arrays' dtypes with NumPy reductions,
as the reference's NumPy backend does.
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft

from . import ptycho_oracle as po


def fourier_clean(array, cutoff=0.66, mask=None, rolloff=0, float_dtype=np.float32):
    """``pypty/utils.py:102-150``: band limit over axes 0 and 1."""
    if cutoff is None and mask is None:
        return array
    shape = array.shape
    if mask is None:
        fx = sfft.fftshift(np.fft.fftfreq(shape[1]))          # utils.py:129-131 (float64)
        fy = sfft.fftshift(np.fft.fftfreq(shape[0]))
        gx, gy = np.meshgrid(fx, fy, indexing="xy")
        r = gx ** 2 + gy ** 2
        max_r = 0.5 * cutoff                                   # utils.py:133
        mask = (r <= max_r ** 2).astype(float_dtype)
        if rolloff != 0:                                       # utils.py:135-137
            r0 = (0.5 * (cutoff - rolloff)) ** 2
            sel = r > r0
            mask[sel] *= 0.5 * (1 + np.cos(3.141592654 * (r - r0) / (max_r ** 2 - r0)))[sel]
    ff = sfft.fftshift(sfft.fft2(array, axes=(0, 1)), axes=(0, 1))
    extra = (None,) * (len(shape) - 2)
    ff = ff * mask[(slice(None), slice(None)) + extra]
    return sfft.ifft2(sfft.ifftshift(ff, axes=(0, 1)), axes=(0, 1))


def wolfe_1(value, new_value, d_value, step, wolfe_c1=0.5):
    return new_value <= value + wolfe_c1 * step * d_value     # utils.py:348


def wolfe_2(d_value, new_d_value, wolfe_c2=0.9):
    return -1 * new_d_value <= -1 * d_value * wolfe_c2         # utils.py:368


def make_states_orthogonal(p):
    """``pypty/objective.py:1133-1141`` for a (W, W, Mp) probe."""
    p = p.copy()
    for i in range(p.shape[-1]):
        for j in range(i):
            p[:, :, i] = p[:, :, i] - p[:, :, j] * (np.sum(np.conjugate(p[:, :, j]) * p[:, :, i])) / (
                1e-10 + np.sum(np.abs(p[:, :, j]) ** 2))
    return p


class Problem:
    """Everything ``loss_and_direction`` needs besides (obj, probe, pos_correction)."""

    def __init__(self, positions, distance, edge_mult, measured, algorithm, wavelength, px, py,
                 damping_cutoff, sequence, loss_weight, compute_batch,
                 float_dtype=np.float32, complex_dtype=np.complex64):
        self.positions, self.distance, self.edge_mult = positions, distance, edge_mult
        self.measured, self.algorithm, self.wavelength = measured, algorithm, wavelength
        self.px, self.py, self.damping_cutoff = px, py, damping_cutoff
        self.sequence, self.loss_weight, self.compute_batch = sequence, loss_weight, compute_batch
        self.f, self.c = float_dtype, complex_dtype

    def lad(self, obj, probe, corr, step_probe, step_obj, step_pos):
        # smooth_rolloff_loss = 0 (iterative.py:476)
        return po.loss_and_direction(obj, probe, self.positions, corr, self.distance, self.edge_mult,
                                     self.measured, self.algorithm, self.wavelength, step_probe, step_obj,
                                     step_pos, self.px, self.py, self.damping_cutoff, 0.0, self.sequence,
                                     self.loss_weight, self.compute_batch, float_dtype=self.f,
                                     complex_dtype=self.c)


class BfgsOracle:
    """State of ``history_bfgs`` plus the refined arrays; ``update`` is one ``bfgs_update``."""

    def __init__(self, problem: Problem, obj, probe, corr):
        self.p = problem
        self.obj, self.probe, self.corr = obj.copy(), probe.copy(), corr.copy()
        self.reset()

    def reset(self):
        """``pypty/iterative.py:1055-1103`` (only the entries of the supported variables)."""
        self.h = dict(obj_s=[], probe_s=[], pos_s=[], obj_y=[], probe_y=[], pos_y=[], rho=[],
                      prev=None, empty=True, g_obj=1, g_probe=1, g_pos=1)

    def update(self, step_obj=True, step_probe=True, step_pos=False, cutoff=np.float32(2 / 3),
               extra_cut=np.float32(0.005), rolloff=np.float32(0), lazy_clean=False, orthogonal=False,
               c1=0.5, c2=0.9, max_count=None, reduce_factor=np.float32(0.1), optimism=3, threshold=1e-20,
               hist_length=10, actual_step=1):
        """One call of ``bfgs_update`` (``pypty/iterative.py:440-1049``); returns
        (total_loss, sse, actual_step, count, d_value, new_d_value, accepted)."""
        h = self.h
        cc = cutoff - extra_cut
        clean = (lambda a: fourier_clean(a, cutoff=cc, rolloff=rolloff, float_dtype=self.p.f).astype(a.dtype))
        # iterative.py:491-514
        if step_probe:
            if self.probe.shape[-1] > 1 and orthogonal:
                self.probe = make_states_orthogonal(self.probe)
            self.probe = clean(self.probe)
        if step_obj and not lazy_clean:
            self.obj = clean(self.obj)
        if h["empty"]:
            loss, sse, og, pg, posg = self.p.lad(self.obj, self.probe, self.corr, step_probe, step_obj, step_pos)
            if step_probe:
                pg = clean(pg)
            if not lazy_clean and step_obj:
                og = clean(og)
            # iterative.py:562-571
            u_obj = -1 * og if step_obj else 0
            d_val_obj = 2 * np.sum(np.abs(u_obj) ** 2)
            if d_val_obj == 0:
                d_val_obj = 1
            u_probe = -1 * pg * d_val_obj / (2 * np.sum(np.abs(pg) ** 2)) if step_probe else 0
            u_pos = -1 * posg * d_val_obj / (np.sum(posg ** 2)) if step_pos else 0
            h["empty"] = False
        else:
            loss, sse, og, pg, posg = h["prev"]
            if step_probe:
                pg = clean(pg)
            # two-loop recursion, iterative.py:583-681
            q_obj = 1 * og if step_obj else 0
            q_probe = 1 * pg if step_probe else 0
            q_pos = 1 * posg if step_pos else 0
            alphas = []
            for i in range(len(h["rho"]) - 1, -1, -1):
                siq = 0
                if step_obj:
                    siq += 2 * np.sum(np.real(h["obj_s"][i] * np.conjugate(q_obj)))
                if step_probe:
                    siq += 2 * np.sum(np.real(h["probe_s"][i] * np.conjugate(q_probe)))
                if step_pos:
                    siq += np.sum(h["pos_s"][i] * q_pos)
                a = h["rho"][i] * siq
                alphas.append(a)
                if step_obj:
                    q_obj -= a * h["obj_y"][i]
                if step_probe:
                    q_probe -= a * h["probe_y"][i]
                if step_pos:
                    q_pos -= a * h["pos_y"][i]
            alphas = alphas[::-1]
            for on, key in ((step_obj, "g_obj"), (step_probe, "g_probe"), (step_pos, "g_pos")):
                if on:
                    gm = h[key]
                    if gm != 0 and gm == gm:
                        if key == "g_obj":
                            q_obj *= gm
                        elif key == "g_probe":
                            q_probe *= gm
                        else:
                            q_pos *= gm
            for i in range(len(h["rho"])):
                yr = 0
                if step_obj:
                    yr += 2 * np.sum(np.real(h["obj_y"][i] * np.conjugate(q_obj)))
                if step_probe:
                    yr += 2 * np.sum(np.real(h["probe_y"][i] * np.conjugate(q_probe)))
                if step_pos:
                    yr += np.sum(h["pos_y"][i] * q_pos)
                beta = alphas[i] - h["rho"][i] * yr
                if step_obj:
                    q_obj += beta * h["obj_s"][i]
                if step_probe:
                    q_probe += beta * h["probe_s"][i]
                if step_pos:
                    q_pos += beta * h["pos_s"][i]
            u_obj = -1 * q_obj if step_obj else 0
            u_probe = -1 * q_probe if step_probe else 0
            u_pos = -1 * q_pos if step_pos else 0
            if not lazy_clean and step_obj:
                u_obj = clean(u_obj)
        def dval(uo, up, us, go, gp, gs):      # iterative.py:684-690, 811-817
            d = 0
            if step_obj:
                d += 2 * np.sum(np.real(np.conjugate(uo) * go))
            if step_probe:
                d += 2 * np.sum(np.real(np.conjugate(up) * gp))
            if step_pos:
                d += np.sum(us * gs)
            return d

        d_value = dval(u_obj, u_probe, u_pos, og, pg, posg)
        if d_value >= 0:                        # iterative.py:691-724
            u_obj = -1 * og if step_obj else 0
            u_probe = -1 * pg if step_probe else 0
            u_pos = -1 * posg if step_pos else 0
            if step_obj and h["g_obj"] > 0 and h["g_obj"] == h["g_obj"]:
                u_obj = u_obj * h["g_obj"]
            if step_probe and h["g_probe"] > 0 and h["g_probe"] == h["g_probe"]:
                u_probe = u_probe * h["g_probe"]
            if step_pos and h["g_pos"] > 0 and h["g_pos"] == h["g_pos"]:
                u_pos = u_pos * h["g_pos"]
            d_value = dval(u_obj, u_probe, u_pos, og, pg, posg)
        # line search, iterative.py:733-837
        count = -1
        while True:
            count += 1
            if step_obj:
                new_obj = self.obj + actual_step * u_obj
                if not lazy_clean:
                    new_obj = clean(new_obj)
            else:
                new_obj = self.obj
            new_probe = self.probe + actual_step * u_probe if step_probe else self.probe
            new_corr = self.corr + actual_step * u_pos if step_pos else self.corr
            n_loss, n_sse, nog, npg, nposg = self.p.lad(new_obj, new_probe, new_corr, step_probe, step_obj,
                                                        step_pos)
            if step_probe:
                npg = clean(npg)
            if not lazy_clean and step_obj:
                nog = clean(nog)
            new_d_value = dval(u_obj, u_probe, u_pos, nog, npg, nposg)
            w1 = wolfe_1(loss, n_loss, d_value, actual_step, c1)
            w2 = wolfe_2(d_value, new_d_value, c2)
            if w1 and w2:
                break
            if not w1 and w2:
                actual_step *= reduce_factor
            if not w2 and w1:
                actual_step *= optimism
            if not (w2 or w1):
                actual_step = type(actual_step)(10 ** (np.random.uniform(0, 20) - 20))
            if max_count is not None and count > max_count:
                break
            if actual_step < threshold:
                break
        if not w1:                              # iterative.py:838-844
            self.reset()
            return loss, sse, actual_step, count, d_value, new_d_value, False
        # history, iterative.py:849-931
        if step_obj:
            h["obj_s"].append(actual_step * u_obj)
            h["obj_y"].append(nog - og)
        if step_probe:
            h["probe_s"].append(actual_step * u_probe)
            h["probe_y"].append(npg - pg)
        if step_pos:
            h["pos_s"].append(actual_step * u_pos)
            h["pos_y"].append(nposg - posg)
        h["prev"] = (n_loss, n_sse, nog, npg, nposg)
        tot = 0
        if step_obj:
            yy = np.sum(np.abs(h["obj_y"][-1]) ** 2)
            ys = 2 * np.sum(np.real(h["obj_y"][-1] * np.conjugate(h["obj_s"][-1])))
            h["g_obj"] = ys / yy
            tot += ys
        if step_probe:
            yy = np.sum(np.abs(h["probe_y"][-1]) ** 2)
            ys = 2 * np.sum(np.real(h["probe_y"][-1] * np.conjugate(h["probe_s"][-1])))
            h["g_probe"] = ys / yy
            tot += ys
        if step_pos:
            yy = np.sum(h["pos_y"][-1] ** 2)
            ys = np.sum(h["pos_y"][-1] * h["pos_s"][-1])
            h["g_pos"] = ys / yy
            tot += ys
        h["rho"].append(1 / tot)
        while len(h["rho"]) > hist_length:
            for k in ("obj_s", "probe_s", "pos_s", "obj_y", "probe_y", "pos_y"):
                if h[k]:
                    h[k].pop(0)
            h["rho"].pop(0)
        self.probe = 1 * new_probe
        self.obj = 1 * new_obj
        if step_pos:
            self.corr = 1 * new_corr
        return loss, sse, actual_step, count, d_value, new_d_value, True
