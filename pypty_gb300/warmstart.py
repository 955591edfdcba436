"""Learned warm start for the multislice reconstruction (no counterpart in the reference).

A 4-level U-Net (base 32 channels: 32 / 64 / 128 / 256; two 3x3 convolutions + ReLU per level,
2x2 average pooling down, nearest upsampling + skip concatenation up, a 1x1 output convolution)
maps per-position centre-of-mass x / y and virtual-bright-field maps (the scan's 32 x 32 grid,
placed bilinearly at the probe centres of the object frame) to the Z-slice phase stack. Every
layer runs in this library's kernels (``csrc/unet.cu``: BF16 activations, FP32 accumulation and
weights, deterministic weight gradients, Adam); training data are specimens of random Gaussian
atoms (peak phase 0.1-1.5 rad for atomic numbers 6-79, linear) simulated through this library's
own multislice forward (``pty_simulate_patterns``) with Poisson noise.

The network covers the object region the scan illuminates (``frame`` x ``frame`` pixels from the
origin: scan extent plus one window); outside it the start stays flat. The flat start
(``obj = ones``, ``pypty/iterative.py:131``) stays the fallback and the yardstick:
``reconstruct`` runs the same GPU-resident L-BFGS loop (``optim.LBFGS``) from either start and
records the phase RMSE against the ground truth after every epoch.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .engine import Engine, Geometry, make_problem
from .optim import LBFGS, LineSearchConfig

BF16 = torch.bfloat16


def _st(dev):
    return torch.cuda.current_stream(dev).cuda_stream


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _ck(rc, what):
    _lib.check(rc, what)


class Conv3:
    """3x3 convolution + ReLU with FP32 weights (He initialisation)."""

    def __init__(self, ci, co, dev, gen):
        std = (2.0 / (9 * ci)) ** 0.5
        self.w = (torch.randn((co, ci, 3, 3), generator=gen) * std).to(dev)
        self.b = torch.zeros(co, device=dev)
        self.ci, self.co = ci, co
        self.gw, self.gb = torch.zeros_like(self.w), torch.zeros_like(self.b)

    def params(self):
        return [(self.w, self.gw), (self.b, self.gb)]


class UNet:
    """The warm-start network; ``forward`` keeps the activations ``backward`` needs."""

    def __init__(self, in_ch=3, out_ch=20, base=32, levels=4, device="cuda", seed=0):
        self.dev = torch.device(device)
        gen = torch.Generator().manual_seed(seed)
        self.in_ch, self.out_ch, self.levels = in_ch, out_ch, levels
        self.cin = 8                                         # input channels padded to the 8-channel chunk
        ch = [base * 2 ** l for l in range(levels)]
        self.ch = ch
        self.enc = []
        cprev = self.cin
        for l in range(levels):
            self.enc.append((Conv3(cprev, ch[l], self.dev, gen), Conv3(ch[l], ch[l], self.dev, gen)))
            cprev = ch[l]
        self.dec = {}
        for l in range(levels - 2, -1, -1):
            self.dec[l] = (Conv3(ch[l] + ch[l + 1], ch[l], self.dev, gen), Conv3(ch[l], ch[l], self.dev, gen))
        std = (1.0 / ch[0]) ** 0.5
        self.wout = (torch.randn((out_ch, ch[0]), generator=gen) * std).to(self.dev)
        self.bout = torch.zeros(out_ch, device=self.dev)
        self.gwout, self.gbout = torch.zeros_like(self.wout), torch.zeros_like(self.bout)
        self.adam = None
        self.t = 0

    def params(self):
        ps = []
        for a, b in self.enc:
            ps += a.params() + b.params()
        for l in sorted(self.dec):
            a, b = self.dec[l]
            ps += a.params() + b.params()
        ps += [(self.wout, self.gwout), (self.bout, self.gbout)]
        return ps

    # ------------------------------------------------------------------ layers
    def _conv(self, x, conv, N, H, W, relu=True):
        out = torch.empty((N, conv.co, H, W), dtype=BF16, device=self.dev)
        _ck(_lib.lib().pty_nn_conv3x3(_p(x), _p(conv.w), _p(conv.b), _p(out), N, conv.ci, conv.co, H, W, int(relu), 0,
                                      _st(self.dev)), "pty_nn_conv3x3")
        return out

    def _conv_back(self, dy, x, y, conv, N, H, W, need_dx=True):
        """dy: gradient at the post-ReLU output y; accumulates nothing, writes conv.gw / gb."""
        lib, st = _lib.lib(), _st(self.dev)
        _ck(lib.pty_nn_relu_mask(_p(dy), _p(y), dy.numel(), st), "pty_nn_relu_mask")
        n = ctypes.c_int64(0)
        _ck(lib.pty_nn_conv3x3_wgrad_workspace_floats(N, conv.ci, conv.co, H, W, ctypes.byref(n)), "wgrad ws")
        ws = self._ws(int(n.value))
        _ck(lib.pty_nn_conv3x3_wgrad(_p(dy), _p(x), _p(conv.gw), _p(conv.gb), N, conv.ci, conv.co, H, W, _p(ws), st),
            "pty_nn_conv3x3_wgrad")
        if not need_dx:
            return None
        dx = torch.empty((N, conv.ci, H, W), dtype=BF16, device=self.dev)
        _ck(lib.pty_nn_conv3x3(_p(dy), _p(conv.w), None, _p(dx), N, conv.co, conv.ci, H, W, 0, 1, st),
            "pty_nn_conv3x3 (data gradient)")
        return dx

    def _ws(self, nfloat):
        if getattr(self, "_wsbuf", None) is None or self._wsbuf.numel() < nfloat:
            self._wsbuf = torch.empty(max(nfloat, 1), dtype=torch.float32, device=self.dev)
        return self._wsbuf

    def _pool(self, x, N, C, H, W):
        y = torch.empty((N, C, H // 2, W // 2), dtype=BF16, device=self.dev)
        _ck(_lib.lib().pty_nn_avgpool2(_p(x), _p(y), N * C, H, W, 0, _st(self.dev)), "pty_nn_avgpool2")
        return y

    # ------------------------------------------------------------------ network
    def forward(self, x):
        """x: (N, 8, H, W) BF16 -> (N, out_ch, H, W) BF16 phase."""
        N, _, H, W = x.shape
        lib, st = _lib.lib(), _st(self.dev)
        acts = {"x": x}
        cur, h, w = x, H, W
        for l, (a, b) in enumerate(self.enc):
            if l > 0:
                cur = self._pool(cur, N, self.ch[l - 1], h, w)
                h, w = h // 2, w // 2
                acts["p%d" % l] = cur
            ya = self._conv(cur, a, N, h, w)
            yb = self._conv(ya, b, N, h, w)
            acts["e%da" % l], acts["e%d" % l] = ya, yb
            cur = yb
        for l in range(self.levels - 2, -1, -1):
            a, b = self.dec[l]
            h, w = h * 2, w * 2
            cl, cu = self.ch[l], self.ch[l + 1]
            cat = torch.empty((N, cl + cu, h, w), dtype=BF16, device=self.dev)
            skip = acts["e%d" % l]
            _ck(lib.pty_nn_channel_copy(_p(skip), _p(cat), N, cl, cl + cu, 0, h * w, 1, st), "concat")
            _ck(lib.pty_nn_upsample2(_p(cur), _p(cat), N, cu, cl + cu, cl, h // 2, w // 2, 0, st), "upsample")
            ya = self._conv(cat, a, N, h, w)
            yb = self._conv(ya, b, N, h, w)
            acts["cat%d" % l], acts["d%da" % l], acts["d%d" % l] = cat, ya, yb
            cur = yb
        out = torch.empty((N, self.out_ch, H, W), dtype=BF16, device=self.dev)
        _ck(lib.pty_nn_conv1x1(_p(cur), _p(self.wout), _p(self.bout), _p(out), N, self.ch[0], self.out_ch, H * W, st),
            "pty_nn_conv1x1")
        self._acts, self._shape = acts, (N, H, W)
        return out

    def backward(self, dout):
        """dout: dL/d(output) (N, out_ch, H, W) BF16; fills every parameter gradient."""
        lib, st = _lib.lib(), _st(self.dev)
        acts = self._acts
        N, H, W = self._shape
        sizes = {l: (H >> l, W >> l) for l in range(self.levels)}
        top = acts["d0"]
        n = ctypes.c_int64(0)
        _ck(lib.pty_nn_conv1x1_workspace_floats(N, self.ch[0], self.out_ch, H * W, ctypes.byref(n)), "1x1 ws")
        ws = self._ws(int(n.value))
        dcur = torch.empty_like(top)
        _ck(lib.pty_nn_conv1x1_backward(_p(dout), _p(top), _p(self.wout), _p(dcur), _p(self.gwout), _p(self.gbout), N,
                                        self.ch[0], self.out_ch, H * W, _p(ws), st), "pty_nn_conv1x1_backward")
        # decoder, full resolution first: dcur is the gradient at the decoder output d_l
        dskip = {}
        for l in range(0, self.levels - 1):
            a, b = self.dec[l]
            h, w = sizes[l]
            cl, cu = self.ch[l], self.ch[l + 1]
            da = self._conv_back(dcur, acts["d%da" % l], acts["d%d" % l], b, N, h, w)
            dcat = self._conv_back(da, acts["cat%d" % l], acts["d%da" % l], a, N, h, w)
            ds = torch.empty((N, cl, h, w), dtype=BF16, device=self.dev)
            _ck(lib.pty_nn_channel_copy(_p(dcat), _p(ds), N, cl, cl + cu, 0, h * w, 0, st), "concat back")
            dskip[l] = ds
            du = torch.empty((N, cu, h // 2, w // 2), dtype=BF16, device=self.dev)
            _ck(lib.pty_nn_upsample2(_p(dcat), _p(du), N, cu, cl + cu, cl, h // 2, w // 2, 1, st), "upsample back")
            dcur = du     # gradient at d_{l+1} (the bottleneck output e_{levels-1} after the last level)
        # encoder, bottleneck first: dcur is the gradient at e_l
        for l in range(self.levels - 1, -1, -1):
            a, b = self.enc[l]
            h, w = sizes[l]
            if l < self.levels - 1:
                _ck(lib.pty_nn_add(_p(dcur), _p(dskip[l]), dcur.numel(), st), "skip add")
            xin = acts["p%d" % l] if l > 0 else acts["x"]
            da = self._conv_back(dcur, acts["e%da" % l], acts["e%d" % l], b, N, h, w)
            dx = self._conv_back(da, xin, acts["e%da" % l], a, N, h, w, need_dx=l > 0)
            if l > 0:
                dp = torch.empty((N, self.ch[l - 1], 2 * h, 2 * w), dtype=BF16, device=self.dev)
                _ck(lib.pty_nn_avgpool2(_p(dx), _p(dp), N * self.ch[l - 1], 2 * h, 2 * w, 1, st), "pool back")
                dcur = dp

    def step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        """Adam (Kingma & Ba 2015) over every parameter."""
        lib, st = _lib.lib(), _st(self.dev)
        ps = self.params()
        if self.adam is None:
            self.adam = [(torch.zeros_like(p), torch.zeros_like(p)) for p, _ in ps]
        self.t += 1
        lr_t = lr * (1 - b2 ** self.t) ** 0.5 / (1 - b1 ** self.t)
        for (p, g), (m, v) in zip(ps, self.adam):
            _ck(lib.pty_nn_adam(_p(p), _p(g), _p(m), _p(v), p.numel(), lr_t, b1, b2, eps, st), "pty_nn_adam")


def mse(pred, target):
    """(loss, dpred): mean squared error of BF16 pred against float target (FP64 sum)."""
    dev = pred.device
    dpred = torch.empty_like(pred)
    part = torch.empty(256, dtype=torch.float64, device=dev)
    _ck(_lib.lib().pty_nn_mse(_p(pred), _p(target), _p(dpred), _p(part), pred.numel(), _st(dev)), "pty_nn_mse")
    return part.sum() / pred.numel(), dpred


# ---------------------------------------------------------------------- data
@dataclass
class Scene:
    """Fixed experiment of the warm-start study: probe, scan and the simulation problem."""
    problem: object
    geometry: Geometry
    probe: torch.Tensor
    n_scan: int
    step_px: float
    W: int
    Z: int
    obj_n: int
    frame: int
    px: float
    wavelength: float


def make_scene(eng: Engine, W=128, Z=20, Mp=3, obj_n=512, n_scan=32, step_A=0.4, px=0.1, kV=300.0, alpha=30.0,
               defocus=50.0, dz=2.0, dose=1e5, seed=0, algorithm="lsq_sqrt") -> Scene:
    """The 128-px / 20-slice / 3-mode experiment of the multislice benchmark (regular scan).

    The reconstructions of the study use the amplitude loss by default: from an exactly flat
    object the model's dark-field intensity is FFT rounding noise (down to denormals in
    focus), where the Poisson loss's dL/dI = (I - M) / I overflows for any measured count,
    in the reference's float32 arithmetic as here; the amplitude loss stays finite there."""
    from . import synth
    probe = synth.make_probe(W, px, kV, alpha, defocus, Mp, [0.6, 0.3, 0.1][:Mp], dose)
    step = step_A / px
    pos = synth.raster_positions(n_scan, n_scan, step)
    ipos, corr = synth.split_positions(pos)
    geo = Geometry.make(ipos, corr)
    lam = synth.wavelength_A(kV)
    prob = make_problem(W, (obj_n, obj_n, Z, 1), Mp, geo, algorithm=algorithm, wavelength=lam, pixel_size_x=px,
                        pixel_size_y=px, slice_distance=dz, compute_batch=256, step_obj=True, step_probe=False,
                        step_pos=False)
    frame = int(np.ceil((ipos.max() + W) / 32.0) * 32)
    return Scene(prob, geo, torch.from_numpy(probe).to(eng.device), n_scan, step, W, Z, obj_n, frame, px, lam)


def specimen(scene: Scene, rng, eng: Engine, n_atoms=150, sigma_A=0.3):
    """Random atoms per slice (Z 6-79 -> peak phase 0.1-1.5 rad, linear) on the device:
    returns (phase (Z, n, n) float32, obj (n, n, Z, 1) complex64)."""
    n, Z = scene.obj_n, scene.Z
    atoms = np.empty((Z, n_atoms, 3), dtype=np.float32)
    atoms[:, :, 0] = rng.uniform(0, n, (Z, n_atoms))
    atoms[:, :, 1] = rng.uniform(0, n, (Z, n_atoms))
    zn = rng.integers(6, 80, (Z, n_atoms))
    atoms[:, :, 2] = 0.1 + (zn - 6) * (1.4 / 73.0)
    a = torch.from_numpy(atoms).to(eng.device)
    phase = torch.empty((Z, n, n), dtype=torch.float32, device=eng.device)
    obj = torch.empty((n, n, Z, 1), dtype=torch.complex64, device=eng.device)
    _ck(_lib.lib().pty_atom_slices(_p(a), n_atoms, n, n, Z, float(sigma_A / scene.px), _p(phase), _p(obj),
                                   _st(eng.device)), "pty_atom_slices")
    return phase, obj


def measure(scene: Scene, obj, eng: Engine, gen):
    """Simulated detector patterns with Poisson noise (N, W, W) float32."""
    sim = eng.simulate(scene.problem, obj, scene.probe, scene.geometry)
    return torch.poisson(sim.clamp_min(0), generator=gen).contiguous()


def maps(scene: Scene, patterns, eng: Engine, r_bf=None):
    """(3, n_scan, n_scan): centre of mass x, y and bright-field disk sum per position."""
    n = patterns.shape[0]
    out = torch.empty((n, 3), dtype=torch.float32, device=eng.device)
    W = scene.W
    if r_bf is None:
        # the aperture radius in detector pixels: alpha / lambda / (1 / (W px))
        r_bf = 0.030 / scene.wavelength * W * scene.px
    _ck(_lib.lib().pty_virtual_detectors(_p(patterns), n, W, float(r_bf), _p(out), _st(eng.device)),
        "pty_virtual_detectors")
    return out.reshape(scene.n_scan, scene.n_scan, 3).permute(2, 0, 1).contiguous()


def network_input(scene: Scene, m, stats, dev):
    """Normalised maps (N, 3, s, s) placed at the probe centres of the frame: (N, 8, F, F) BF16."""
    mean, std = stats
    x = ((m - mean[None, :, None, None]) / std[None, :, None, None]).contiguous()
    N, F = x.shape[0], scene.frame
    out = torch.empty((N, 8, F, F), dtype=BF16, device=dev)
    off = scene.W / 2.0
    _ck(_lib.lib().pty_nn_bilinear(_p(x), _p(out), N, 3, 8, scene.n_scan, scene.n_scan, F, F, off, off,
                                   float(scene.step_px), float(scene.step_px), _st(dev)), "pty_nn_bilinear")
    return out


def lowpass_target(phase_frame, cutoff, eng: Engine):
    """The part of a (Z, F, F) phase stack the maps can predict: each slice band-limited to
    ``cutoff`` (fraction of Nyquist) with the library's fourier_clean kernel."""
    from .optim import fourier_clean_
    z = phase_frame.permute(1, 2, 0).contiguous().to(torch.complex64)      # (F, F, Z)
    fourier_clean_(z, cutoff, 0.0, out=z, engine=eng)
    return z.real.permute(2, 0, 1).contiguous()


def predictable_target(phase_frame, cutoff, eng: Engine):
    """E[phase_z | maps]: the maps see the depth-integrated phase blurred by the probe, and the
    slices of a random specimen are independent, so the predictable part of every slice is the
    band-limited depth average (each slice's own deviation from it is not predictable)."""
    lp = lowpass_target(phase_frame, cutoff, eng)
    return lp.mean(dim=0, keepdim=True).expand_as(lp).contiguous()


def make_dataset(scene: Scene, n, eng: Engine, seed, target_cutoff=0.1, n_atoms=150):
    """n specimens of ``n_atoms`` atoms per slice: input maps (n, 3, s, s) and target phases
    (n, Z, F, F) on the frame: the conditional-mean target ``predictable_target`` (the scan
    samples every ``step`` pixels and the probe blurs the depth-integrated phase)."""
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=eng.device).manual_seed(seed)
    F = scene.frame
    xs = torch.empty((n, 3, scene.n_scan, scene.n_scan), device=eng.device)
    ys = torch.empty((n, scene.Z, F, F), device=eng.device)
    for i in range(n):
        phase, obj = specimen(scene, rng, eng, n_atoms=n_atoms)
        pat = measure(scene, obj, eng, gen)
        xs[i] = maps(scene, pat, eng)
        ys[i] = predictable_target(phase[:, :F, :F], target_cutoff, eng)
    return xs, ys


def train(net: UNet, scene: Scene, xs, ys, stats, epochs=10, batch=4, lr=1e-3, seed=0, log=None):
    """Adam on the mean squared error of the standardised target phase (the target's mean and
    standard deviation are kept in ``net.target_stats`` and undone by ``predict``); returns the
    per-epoch mean loss (in units of the target variance)."""
    n = xs.shape[0]
    t_mean, t_std = float(ys.mean()), float(ys.std()) + 1e-12
    net.target_stats = (t_mean, t_std)
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(n)
        tot = 0.0
        for b0 in range(0, n - batch + 1, batch):
            idx = torch.from_numpy(order[b0:b0 + batch]).to(xs.device)
            x = network_input(scene, xs[idx], stats, net.dev)
            pred = net.forward(x)
            loss, d = mse(pred, ((ys[idx] - t_mean) / t_std).contiguous())
            net.backward(d)
            net.step(lr)
            tot += float(loss)
        hist.append(tot / max(1, n // batch))
        if log:
            log("epoch %d loss %.5f" % (ep, hist[-1]))
    return hist


def predict(net: UNet, scene: Scene, m, stats):
    """Phase stack (Z, F, F) predicted from the maps m (3, s, s)."""
    x = network_input(scene, m[None], stats, net.dev)
    t_mean, t_std = getattr(net, "target_stats", (0.0, 1.0))
    return net.forward(x)[0].float() * t_std + t_mean


def phase_rmse(obj, truth_phase, region, projected=False, depth_mean=False):
    """RMSE (rad) of the slice phases against the truth over region = (y0, y1, x0, x1), after
    removing each slice's mean difference (a constant phase per slice leaves every pattern
    unchanged, so it is not recoverable). projected=True: of the phase summed over the slices
    (the depth-integrated phase); depth_mean=True: of the phase averaged over the slices (the
    projected phase / Z, on the scale of one slice). The data determine these far better than
    the distribution over slices much thinner than the probe's depth of field (~ lambda /
    alpha^2: 22 A at 300 kV and 30 mrad, against 2 A slices)."""
    y0, y1, x0, x1 = region
    o = obj[y0:y1, x0:x1, :, 0]                          # (h, w, Z)
    t = truth_phase[:, y0:y1, x0:x1].permute(1, 2, 0)
    d = torch.angle(o * torch.exp(-1j * t.to(torch.complex64)))
    if projected:
        d = d.sum(dim=2, keepdim=True)
    elif depth_mean:
        d = d.mean(dim=2, keepdim=True)
    d = d - d.mean(dim=(0, 1), keepdim=True)
    return float(torch.sqrt((d.double() ** 2).mean()))


def reconstruct(scene: Scene, measured, truth_phase, obj0, eng: Engine, epochs=60, target=0.02, region=None,
                time_budget=None):
    """GPU-resident L-BFGS (object only, probe and positions known) from obj0. Returns the list
    of (seconds, per-slice RMSE, depth-mean RMSE) after every epoch and the time at which the
    depth-mean RMSE reached ``target`` (None if it did not; the run stops there, or after
    ``epochs`` epochs or ``time_budget`` seconds). The clock runs over the reconstruction only;
    the RMSE evaluation is excluded."""
    corr = torch.from_numpy(np.ascontiguousarray(scene.geometry.pos_correction)).to(eng.device)
    cfg = LineSearchConfig(update_obj=True, update_probe=False, update_pos=False, wolfe_c1=0.1, max_count=20)
    opt = LBFGS(scene.problem, scene.geometry, measured, obj0.clone(), scene.probe, corr, cfg, engine=eng)
    np.random.seed(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    curve, hit = [], None
    # first step from an empty history: scale -grad so that the largest object change is 0.05
    # (the reference leaves the first step to the user, e.g. update_step_bfgs = 8.1e-9 if epoch == 0)
    _, og, _, _ = eng.loss_and_direction(scene.problem, opt.obj, scene.probe, scene.geometry, measured,
                                         pos_correction=corr)
    step0 = 0.05 / max(float(og.abs().max()), 1e-30)
    paused = 0.0
    retries = 0
    for ep in range(epochs):
        try:
            opt.step(step0 if not opt.history else 1)
        except ValueError:      # a diverging trial (NaN loss)
            # the first step is retried 10x and 100x smaller (for either start alike, as a user
            # picks a small first step); later failures end the run
            if opt.history or retries >= 2:
                break
            retries += 1
            step0 *= 0.1
            opt.reset()
            continue
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        el = t1 - t0 - paused
        es = phase_rmse(opt.obj, truth_phase, region)
        ed = phase_rmse(opt.obj, truth_phase, region, depth_mean=True)
        curve.append((el, es, ed))
        paused += time.perf_counter() - t1
        if hit is None and target is not None and ed <= target:
            hit = el
            break
        if time_budget is not None and el > time_budget:
            break
    return curve, hit


def time_to(curve, level, offset=0.0, index=2, start=None):
    """First time (s) at which an RMSE curve [(s, per-slice, depth-mean)] reaches level in
    column ``index`` (2: depth-mean, 1: per-slice), or None. ``start``: the start's own RMSE,
    which counts at time ``offset`` (a start already below the level needs no epoch)."""
    if start is not None and start <= level:
        return offset
    for row in curve:
        if row[index] <= level:
            return row[0] + offset
    return None
