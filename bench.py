"""Benchmark: scan positions per second of one full loss + adjoint-gradient pass.

Workload (default): the multislice configuration -- 512x512 px x 20 slices object at
0.1 A/px, 128 px probe with 3 incoherent modes (powers 0.6/0.3/0.1) at 300 kV / 30 mrad,
32x32 scan at 0.4 A with U(+-0.2 A) jitter, Poisson loss ("ml"), compute batch 256,
complex64. One step = one call of the loss-and-direction path over all 1024 positions
(forward multislice, far-field Poisson loss, adjoint multislice, object / probe / position
gradients). Inputs are seeded synthetic data: the measured patterns are simulated with the
library's own forward model from the true specimen plus Poisson noise, and the gradient is
evaluated at a half-phase start, so no step is skipped or cached.

`value`   positions/s with object, probe and patterns resident in HBM (device-timed).
`e2e`     positions/s through the public call with host buffers: each step copies object,
          probe and patterns host->device and gradients + loss device->host.
`streamed_patterns` positions/s with the measured patterns left in pinned host memory and
          read in place by the kernels (a dataset larger than HBM), object and probe in HBM.
`roofline` the dominant kernel (fused_multislice) timed live with CUDA events on its
          stream; algorithmic bytes per launch: the path's algorithmic bytes per position
          W^2 (32 Z Mo + 16 Z Mp Mo + 4) (alg_bytes_per_position below: object windows read
          forward and adjoint, gradient read-modify-write, wave stack write + read, measured
          pattern read) times the positions per launch.

The working set of a step (object 42 MB, patterns 67 MB, per-batch wave stack 2 GB) is
far larger than the 129 MB L2, so no explicit L2 flush is needed between steps.

Under torchrun with N GPUs every rank runs the same workload on its own GPU (replicas:
the path needs no collective), `value` is the sum over ranks of positions/s.

`--impl reference` times the reference algorithm on the host cores: the NumPy restatement
in oracle/ (the reference is pure Python and is not installed on the GPU host), on a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (W, Ny, Z, Mp, n_scan, algorithm, batch)
    "multislice": dict(W=128, N_obj=512, Z=20, Mp=3, n_scan=32, algorithm="ml", batch=256,
                       desc="multislice W128 Z20 Mp3 Mo1, 512x512 object, 32x32 jittered scan, ml, batch 256"),
    # the "multislice" workload plus the variants path (near field, tilts, beam current,
    # aberration plates, compressed detectors) timed on it
    "variants": dict(W=128, N_obj=512, Z=20, Mp=3, n_scan=32, algorithm="ml", batch=256, variants=True,
                     desc="multislice W128 Z20 Mp3 Mo1, 512x512 object, 32x32 jittered scan, ml, batch 256; "
                          "variants path timed on the same positions"),
    # same kernels and shapes per position as "multislice", 8x8 positions: for ncu captures
    "multislice-small": dict(W=128, N_obj=512, Z=20, Mp=3, n_scan=8, algorithm="ml", batch=64,
                             desc="multislice W128 Z20 Mp3 Mo1, 512x512 object, 8x8 jittered scan, ml, batch 64"),
    # 256-px windows, 5 modes, 40 slices over a 1024^2 object, 64x64 scan (FP32 FFT path)
    "precision-sweep": dict(W=256, N_obj=1024, Z=40, Mp=5, n_scan=64, algorithm="lsq_sqrt", batch=512, sweep=True,
                            desc="precision sweep W256 Z40 Mp5 Mo1, 1024x1024 object, 64x64 scan, lsq_sqrt, batch 512"),
    # the precision sweep's shapes per position on 8x8 positions and 8 slices: for ncu captures
    "precision-sweep-small": dict(W=256, N_obj=1024, Z=8, Mp=5, n_scan=8, algorithm="lsq_sqrt", batch=64,
                                  sweep=True, desc="precision sweep W256 Z8 Mp5 Mo1, 1024x1024 object, 8x8 scan, "
                                                   "lsq_sqrt, batch 64"),
    # 256-px windows, 8 modes, 60 slices over a 2048^2 object, 128x128 scan, batch 512
    "large-adjoint": dict(W=256, N_obj=2048, Z=60, Mp=8, n_scan=128, algorithm="lsq_sqrt", batch=512,
                          desc="large adjoint W256 Z60 Mp8 Mo1, 2048x2048 object, 128x128 scan, lsq_sqrt, batch 512"),
    # learned warm start: train the U-Net on simulated specimens of the 128-px / 20-slice / 3-mode
    # experiment, then time the reconstruction to 0.02 rad phase RMSE from the learned and the flat start
    "warm-start": dict(W=128, N_obj=512, Z=20, Mp=3, n_scan=32, algorithm="ml", batch=256, warm_start=True,
                       desc="learned warm start: U-Net (4 levels, base 32, BF16) on CoM-x/CoM-y/vBF maps of a "
                            "32x32 scan, 512x512x20 specimens, W128 Mp3"),
    "single-slice": dict(W=64, N_obj=128, Z=1, Mp=1, n_scan=16, algorithm="lsq_sqrt", batch=256,
                         desc="single-slice W64 Z1 Mp1, 128x128 object, 16x16 scan, lsq_sqrt, batch 256"),
}


def alg_bytes_per_position(W, Z, Mp, Mo=1):
    """Algorithmic HBM bytes of one position (complex64 = 8 B, float32 patterns = 4 B):
    W^2 * (32 Z Mo + 16 Z Mp Mo + 4): object windows read forward + adjoint, gradient
    read-modify-write, wave stack write + read, measured pattern read."""
    return W * W * (32 * Z * Mo + 16 * Z * Mp * Mo + 4)


def fused_bytes_per_position(W, Z, Mp, Mo=1):
    """Bytes the fused multislice kernel must move per position: band-limited object
    windows read forward and adjoint (16 Z Mo), wave stack write + read (16 Z Mp Mo),
    one object-gradient contribution window per probe mode written (8 Z Mp Mo; the modes are
    summed in order by the band-limit kernel), measured pattern read (4), per-position
    probe-gradient spectra written (8 Mp)."""
    return W * W * (16 * Z * Mo + 16 * Z * Mp * Mo + 8 * Z * Mp * Mo + 4 + 8 * Mp)


# DRAM bytes (read + write) per position of the fused kernel(s), from one ncu capture each
# (dram__bytes_read.sum + dram__bytes_write.sum of the launch / positions in it); a launch of
# the same shape moves the same bytes per position, so traffic per launch scales by positions:
#   (128, 20, 3): fused_multislice_kernel<128>, multislice-small, 64 positions, 1.7056 GB
#   (256, 8, 5):  fused256_kernel<1> + <2>, precision-sweep-small, 64 positions, 10.674 GB
TRAFFIC_PER_POSITION = {(128, 20, 3): 1.7056e9 / 64, (256, 8, 5): 10.674e9 / 64}


def fft_flops_per_position(W, Z, Mp, Mo=1):
    """5 W^2 log2(W^2) flops per 2D FFT; FFTs per position of the reference algorithm:
    4 Z Mo (object and gradient band limits) + 4 (Z-1) Mp Mo (propagation both ways)
    + 2 Mp Mo (far field both ways) + 3 Mp (probe shift and its adjoint)."""
    n_fft = 4 * Z * Mo + 4 * (Z - 1) * Mp * Mo + 2 * Mp * Mo + 3 * Mp
    return n_fft * 5.0 * W * W * np.log2(W * W)


def build_workload(cfg, seed=0):
    """Seeded specimen, probe and scan for a configuration (host arrays)."""
    from pypty_gb300 import synth
    rng = np.random.default_rng(seed)
    if cfg["W"] == 256:
        px, kV, alpha, df = 0.1, 300.0, 30.0, 80.0
        dz = 1.0 if cfg["Z"] == 40 else 2.0
        atoms = 400 * (cfg["N_obj"] // 1024) ** 2
        truth = synth.gaussian_phase_object(cfg["N_obj"], cfg["N_obj"], cfg["Z"], atoms, 0.3, px, 0.2, 1.0, rng)
        probe = synth.make_probe(cfg["W"], px, kV, alpha, df, cfg["Mp"], 0.6 ** np.arange(cfg["Mp"]), 1e5)
        pos = synth.raster_positions(cfg["n_scan"], cfg["n_scan"], 0.4 / px, 0.2 / px, rng)
        dose = 1e5
    elif cfg["W"] == 128:
        px, kV, alpha, df, dz = 0.1, 300.0, 30.0, 50.0, 2.0
        truth = synth.gaussian_phase_object(cfg["N_obj"], cfg["N_obj"], cfg["Z"], 150, 0.3, px, 0.2, 1.0, rng)
        probe = synth.make_probe(cfg["W"], px, kV, alpha, df, cfg["Mp"], [0.6, 0.3, 0.1][:cfg["Mp"]], 1e5)
        pos = synth.raster_positions(cfg["n_scan"], cfg["n_scan"], 0.4 / px, 0.2 / px, rng)
        dose = 1e5
    else:
        px, kV, alpha, df, dz = 0.2, 200.0, 25.0, 100.0, 1.0
        truth = synth.gaussian_phase_object(cfg["N_obj"], cfg["N_obj"], cfg["Z"], 60, 0.4, px, 0.5, 2.0, rng)
        probe = synth.make_probe(cfg["W"], px, kV, alpha, df, cfg["Mp"], None, 1e4)
        pos = synth.raster_positions(cfg["n_scan"], cfg["n_scan"], 0.5 / px)
        dose = 1e4
    ipos, corr = synth.split_positions(pos)
    obj0 = np.exp(0.5j * np.angle(truth)).astype(np.complex64)
    return dict(truth=truth, obj0=obj0, probe=probe, ipos=ipos, corr=corr, px=px, kV=kV, dz=dz, dose=dose,
                wavelength=synth.wavelength_A(kV), rng=rng)


def simulate_measured(eng, prob, wl, geo):
    """Measured patterns of a workload: the library's forward model at the true specimen
    (float32 mean-over-modes intensities, detector order) plus Poisson noise drawn on the
    device with a generator seeded 1. Returns a (N, W, W) float32 CUDA tensor."""
    import torch
    dev = eng.device
    truth_d = torch.from_numpy(wl["truth"]).to(dev)
    probe_d = torch.from_numpy(wl["probe"]).to(dev)
    sim = eng.simulate(prob, truth_d, probe_d, geo)
    gen = torch.Generator(device=dev).manual_seed(1)
    meas_d = torch.poisson(sim.clamp_min(0), generator=gen).contiguous()
    del truth_d, sim
    return meas_d


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in open(self.file.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(cfg, wl, algorithm, budget_s=15.0, cores=None):
    """The oracle (NumPy restatement of the reference path) on a bounded sample of positions,
    on `cores` host cores (scipy.fft workers; default all): a short calibration call sizes the
    sample so that the timed call takes about `budget_s` seconds. cores=1 is the reference as
    shipped (pypty/fft.py:111-156 passes scipy.fft no workers)."""
    import scipy.fft
    from oracle import ptycho_oracle as orc
    cores = cores or os.cpu_count() or 1
    n_max = wl["ipos"].shape[0]

    def run(n):
        seq = np.arange(n)
        meas = np.zeros((n, cfg["W"], cfg["W"]), np.float32) + 1.0
        t0 = time.perf_counter()
        orc.loss_and_direction(wl["obj0"], wl["probe"], wl["ipos"][:n], wl["corr"][:n], wl["dz"], 1.0, meas,
                               algorithm, wl["wavelength"], 1, 1, 1, wl["px"], wl["px"], 2 / 3, 0.0, seq, 1,
                               cfg["batch"])
        return time.perf_counter() - t0

    with scipy.fft.set_workers(cores):
        n0 = min(4, n_max)
        t_cal = run(n0)
        n = int(max(n0, min(n_max, budget_s * n0 / max(t_cal, 1e-6))))
        dt = run(n)
    return {"value": n / dt, "unit": "positions/s", "cores": cores, "kind": "port",
            "sample": "%d positions of the %s workload (NumPy/SciPy oracle, complex64, %.1f s)" % (
                n, cfg["name"], dt), "seconds": dt, "positions": n}


def run_warm_start(args, cfg):
    """Learned vs flat start (the warm-start configuration): train on simulated specimens, then
    reconstruct held-out specimens with the GPU-resident L-BFGS from both starts and report the
    wall time to 0.02 rad phase RMSE (inference included for the learned start).

    The RMSE that decides is the one of the depth-averaged phase (projected phase / Z, per
    slice scale): the 20 slices are 2 A apart, a tenth of the probe's depth of field (~22 A at
    300 kV and 30 mrad), so their individual phases are not determined by the data and no start
    reaches 0.02 rad per slice; the per-slice RMSE is reported beside it."""
    import torch
    from pypty_gb300 import warmstart as ws
    from pypty_gb300.engine import Engine
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    eng = Engine(dev)
    scene = ws.make_scene(eng, W=cfg["W"], Z=cfg["Z"], Mp=cfg["Mp"], obj_n=cfg["N_obj"], n_scan=cfg["n_scan"])
    t0 = time.perf_counter()
    xs, ys = ws.make_dataset(scene, args.train, eng, seed=100, target_cutoff=0.25)
    torch.cuda.synchronize(dev)
    t_data = time.perf_counter() - t0
    stats = (xs.mean(dim=(0, 2, 3)), xs.std(dim=(0, 2, 3)) + 1e-6)
    net = ws.UNet(in_ch=3, out_ch=cfg["Z"], base=32, levels=4, device=dev, seed=0)
    t0 = time.perf_counter()
    hist = ws.train(net, scene, xs, ys, stats, epochs=args.epochs, batch=4, lr=args.lr)
    torch.cuda.synchronize(dev)
    t_train = time.perf_counter() - t0
    del xs, ys
    rng = np.random.default_rng(999)
    gen = torch.Generator(device=dev).manual_seed(999)
    F = scene.frame
    c0, c1 = int(scene.W / 2), int(scene.geometry.positions.max() + scene.W / 2)
    region = (c0, c1, c0, c1)          # the probe centres' square: every pixel well illuminated
    rows = []
    ws.predict(net, scene, torch.zeros((3, scene.n_scan, scene.n_scan), device=dev), stats)   # warm the path up
    for k in range(args.test):
        phase, obj = ws.specimen(scene, rng, eng)
        meas = ws.measure(scene, obj, eng, gen)
        flat = torch.ones_like(obj)
        torch.cuda.synchronize(dev)
        t_inf0 = time.perf_counter()
        m = ws.maps(scene, meas, eng)
        pred = ws.predict(net, scene, m, stats)                      # (Z, F, F)
        start = torch.ones_like(obj)
        start[:F, :F, :, 0] = torch.exp(1j * pred.permute(1, 2, 0).to(torch.complex64))
        torch.cuda.synchronize(dev)
        t_inf = time.perf_counter() - t_inf0
        tgt = ws.predictable_target(phase[:, :F, :F], 0.25, eng)
        a, b = pred[0, c0:c1, c0:c1].flatten(), tgt[0, c0:c1, c0:c1].flatten()
        row = {"inference_s": round(t_inf, 4), "pred_target_corr": round(float(torch.corrcoef(torch.stack([a, b]))[0, 1]), 4)}
        cf, _ = ws.reconstruct(scene, meas, phase, flat, eng, epochs=args.recon_epochs, region=region, target=None)
        cl, _ = ws.reconstruct(scene, meas, phase, start, eng, epochs=args.recon_epochs, region=region, target=None)
        for key, idx, dm in (("depth_mean", 2, True), ("slices", 1, False)):
            r0f = ws.phase_rmse(flat, phase, region, depth_mean=dm)
            r0l = ws.phase_rmse(start, phase, region, depth_mean=dm)
            levels = {"0.02": 0.02, "0.75_flat0": 0.75 * r0f, "0.5_flat0": 0.5 * r0f}
            row[key] = {"rmse0": {"flat": round(r0f, 4), "learned": round(r0l, 4)},
                        "final": {"flat": round(cf[-1][idx], 4) if cf else None,
                                  "learned": round(cl[-1][idx], 4) if cl else None},
                        "time_to": {name: {"flat": ws.time_to(cf, lv, 0.0, idx, r0f),
                                           "learned": ws.time_to(cl, lv, t_inf, idx, r0l)}
                                    for name, lv in levels.items()}}
        row["flat_curve"] = [(round(c[0], 3), round(c[1], 4), round(c[2], 4)) for c in cf[::5]]
        row["learned_curve"] = [(round(c[0], 3), round(c[1], 4), round(c[2], 4)) for c in cl[::5]]
        rows.append(row)

    def stat(key, level, who):
        v = [r[key]["time_to"][level][who] for r in rows]
        got = [x for x in v if x is not None]
        return {"mean_s": float(np.mean(got)) if len(got) == len(v) else None, "reached": len(got), "of": len(v)}

    summary = {key: {lv: {"flat": stat(key, lv, "flat"), "learned": stat(key, lv, "learned")}
                     for lv in ("0.02", "0.75_flat0", "0.5_flat0")} for key in ("depth_mean", "slices")}
    for key in ("depth_mean", "slices"):
        summary[key]["rmse0"] = {who: float(np.mean([r[key]["rmse0"][who] for r in rows])) for who in ("flat", "learned")}
    v_l, v_f = summary["depth_mean"]["0.02"]["learned"]["mean_s"], summary["depth_mean"]["0.02"]["flat"]["mean_s"]
    line = {"metric": "time to 0.02 rad phase RMSE (depth-averaged phase), learned vs plain init", "impl": "ours",
            "value": v_l, "unit": "s", "higher_is_better": False, "plain_s": v_f,
            "ratio_learned_over_plain": (v_l / v_f) if v_l is not None and v_f else None,
            "summary": summary, "n_gpus": 1, "data": "synthetic", "dtype": "bf16 network, c64 reconstruction",
            "config": {"workload": cfg["desc"], "train_specimens": args.train, "test_specimens": args.test,
                       "epochs": args.epochs, "recon_epochs": args.recon_epochs, "frame_px": F, "region": region,
                       "loss": "lsq_sqrt (amplitude)", "network_target": "depth-mean phase band-limited to 0.25 Nyquist"},
            "train": {"dataset_s": round(t_data, 2), "train_s": round(t_train, 2), "loss": [round(h, 5) for h in hist]},
            "mean_pred_target_corr": float(np.mean([r["pred_target_corr"] for r in rows])),
            "specimens": rows}
    print(json.dumps(line))


def variants_timing(eng, prob, geo, meas_d, obj_d, probe_d, n_pos, steps=3):
    """Device-timed positions/s of pty_loss_and_direction_variants on the benchmark workload
    with each family of variant branches switched on (one warm-up call, `steps` timed calls):
    the far-field layered path itself, near-field propagation, beam tilts (mode 4, one row per
    position, with the tilt gradient), beam current + aberration plates (with gradients), a
    compressed-detector loss on 8 masks, and the measured-data preprocessing."""
    import torch
    from pypty_gb300 import _lib
    dev = obj_d.device
    stream = torch.cuda.current_stream(dev)
    W = prob.window
    N = prob.n_positions
    rng = np.random.default_rng(3)
    tilts = (rng.normal(size=(N, 6)) * 2e-4).astype(np.float32)
    bc = torch.from_numpy((1 + 0.05 * rng.normal(size=N)).astype(np.float32)).to(dev)
    ab = torch.from_numpy((rng.normal(size=(2, 7)) * 5).astype(np.float32)).to(dev)
    marker = torch.from_numpy((np.arange(N) % 2).astype(np.int32)).to(dev)
    masks = torch.from_numpy(rng.uniform(0, 1, (8, W, W)).astype(np.float32)).to(dev)
    coef = torch.from_numpy(rng.uniform(1e3, 2e3, (N, 8)).astype(np.float32)).to(dev)
    cases = {
        "far_field_layered": (prob, meas_d, {}),
        "near_field": (prob, meas_d, dict(recon_type="near_field", defocus=50.0, cs=1e5)),
        "tilts_mode4_grad": (prob, meas_d, dict(tilts=tilts, tilt_mode=4, step_tilts=True)),
        "beam_current_aberrations_grad": (prob, meas_d, dict(beam_current=bc, step_beam_current=True,
                                                            aberrations=ab, aberration_marker=marker,
                                                            step_aberrations=True)),
        "data_preprocessing": (prob, meas_d, dict(data_shift_vector=(2, -1), data_multiplier=1.1)),
    }
    cp = _lib.Problem.from_buffer_copy(prob)
    cp.algorithm = _lib.COMPRESSED_ALGORITHMS["lsq_compressed"]
    cases["compressed_lsq_8_masks"] = (cp, coef, dict(masks=masks))
    out = {"positions": n_pos}
    for name, (pr, meas, kw) in cases.items():
        eng.loss_and_direction_variants(pr, obj_d, probe_d, geo, meas, **kw)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            eng.loss_and_direction_variants(pr, obj_d, probe_d, geo, meas, **kw)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"positions_per_s": round(n_pos / (ms / 1000.0), 1), "ms": round(ms, 2)}
    return out


def precision_sweep(eng, wl, geo, meas_d, obj_d, probe_d, cfg, common, n_sub=512, batch=256):
    """The same loss-and-gradient call with every window DFT on each engine of the layered
    path (pty_loss_and_direction_layered: FP32 register FFT, BF16x3 and BF16x6 tensor-core
    GEMMs) and on the fused FP32 path, over the first n_sub positions: device-timed positions/s
    (one warm-up call, one timed call each). Their errors against the FP64 oracle are measured
    by tests/test_gpu_layered.py and tests/test_gpu_dft_gemm.py."""
    import torch
    from pypty_gb300 import _lib
    from pypty_gb300.engine import Geometry, make_problem
    dev = obj_d.device
    stream = torch.cuda.current_stream(dev)
    W, Z, Mp = cfg["W"], cfg["Z"], cfg["Mp"]
    sub = Geometry.make(geo.positions, geo.pos_correction, np.arange(n_sub))
    kw = dict(common, compute_batch=batch)
    prob = make_problem(W, tuple(obj_d.shape), Mp, sub, step_pos=True, **kw)
    out = {"positions": n_sub, "batch": batch}
    # 2D DFTs per position on the layered path: object and gradient-window band limits, probe
    # shift, forward and adjoint propagation, far field and its adjoint, probe-gradient spectrum
    n_dft = 4 * Z + 4 * (Z - 1) * Mp + 2 * Mp + 2 * Mp
    for name in ("fused_fp32", "fp32_fft", "bf16x3", "bf16x6"):
        def call():
            if name == "fused_fp32":
                return eng.loss_and_direction(prob, obj_d, probe_d, sub, meas_d)
            return eng.loss_and_direction_layered(prob, obj_d, probe_d, sub, meas_d, engine=name)
        call()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with _lib.LaunchProfiler(1 << 16) as prof:
            e0.record(stream)
            res = call()
            e1.record(stream)
            torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        row = {"positions_per_s": round(n_sub / (ms / 1e3), 1), "ms": round(ms, 1),
               "loss": float(res[0][0].item())}
        gemm_ms = prof.ms.get("dft_gemm_bf16x3", 0.0)
        if gemm_ms > 0:
            terms = 2 if name == "bf16x3" else 3
            products = 3 if terms == 2 else 6
            flops = n_sub * n_dft * 2 * products * W * (2 * W) * (2 * W) * 2
            row["dft_gemm_share"] = round(gemm_ms / ms, 3)
            row["tensor_tflops"] = round(flops / (gemm_ms / 1e3) / 1e12, 1)
        out[name] = row
        torch.cuda.empty_cache()
    return out


def optimizer_step(eng, prob, geo, meas_d, obj_d, probe_d, wl, lad_ms, hbm_peak, peak_src, epochs=4):
    """The optimizer around loss_and_direction on the same workload: the full-object band
    limit of a trial point (pty_fourier_clean_apply, timed with CUDA events, HBM roofline over
    its algorithmic bytes: read x and dx, write the result) and whole L-BFGS epochs
    (LBFGS.step, wall time around device work and the per-trial host reads)."""
    import torch
    from pypty_gb300 import _lib
    from pypty_gb300.optim import LBFGS, LineSearchConfig, fourier_clean_
    dev = obj_d.device
    stream = torch.cuda.current_stream(dev)
    cut = np.float32(2 / 3) - np.float32(0.005)
    dx = torch.randn_like(obj_d)
    tmp = torch.empty_like(obj_d)
    for _ in range(3):
        fourier_clean_(obj_d, cut, 0.0, out=tmp, dx=dx, step=0.3, engine=eng)
    torch.cuda.synchronize(dev)
    n = 10
    with _lib.LaunchProfiler(64 * n) as prof:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fourier_clean_(obj_d, cut, 0.0, out=tmp, dx=dx, step=0.3, engine=eng)
        e1.record(stream)
        torch.cuda.synchronize(dev)
    clean_ms = e0.elapsed_time(e1) / n
    clean_bytes = 3 * obj_d.numel() * 8
    clean_gbs = clean_bytes / (clean_ms / 1e3) / 1e9
    passes = {k: round(prof.ms.get(k, 0.0) / n, 4) for k in ("clean_pass_x", "clean_pass_y", "clean_pass_x_inverse")}
    del dx, tmp
    corr_d = torch.from_numpy(np.ascontiguousarray(geo.pos_correction)).to(dev)
    opt = LBFGS(prob, geo, meas_d, obj_d.clone(), probe_d.clone(), corr_d,
                LineSearchConfig(update_obj=True, update_probe=True, update_pos=True, wolfe_c1=0.1, max_count=20),
                engine=eng)
    np.random.seed(0)
    rows = []
    for e in range(epochs):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        # the first step from an empty history is -grad at unit scale: start it small, as the
        # reference's own example schedule does ('update_step_bfgs': tiny if epoch == 0 else 1)
        r = opt.step(1e-6 if e == 0 else 1)
        torch.cuda.synchronize(dev)
        wall = (time.perf_counter() - t0) * 1e3
        n_lad = r.count + 1 + (1 if not rows else 0)
        rows.append(dict(ms=round(wall, 3), lad_calls=n_lad, accepted=r.accepted,
                         overhead_ms=round(wall - n_lad * lad_ms, 3)))
    hist = [rw["overhead_ms"] for rw in rows[1:]] or [rows[0]["overhead_ms"]]
    return {"fourier_clean": {"object": list(obj_d.shape), "ms": round(clean_ms, 4), "achieved": round(clean_gbs, 1),
                              "unit": "GB/s", "alg_bytes": clean_bytes, "frac": round(clean_gbs / hbm_peak, 4),
                              "peak_source": peak_src + " (hbm_gbs)", "pass_ms": passes},
            "lbfgs_epochs": rows,
            "overhead_ms_per_epoch_with_history": round(float(np.mean(hist)), 3),
            "lad_ms": round(lad_ms, 3)}


def max_over_ranks(ms, world, device=None):
    """The job's step time: the slowest rank's (all_reduce MAX; one rank: unchanged)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(n_pos_per_rank, world, ms):
    """Positions/s of the whole job: every rank processes its own replica of the workload
    (independent positions, no data-path collective) in the job's step time."""
    return world * n_pos_per_rank / (ms / 1000.0)


def run_reference(args, cfg):
    """--impl reference: the reference algorithm on the host cores, same metric and config."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = build_workload(cfg)
    # each step times a bounded sample; the whole run stays within a few minutes
    budget = max(2.0, min(15.0, 150.0 / max(args.steps, 1)))
    for _ in range(args.warmup):   # untimed warm-up steps on a short sample
        cpu_baseline(cfg, wl, cfg["algorithm"], budget_s=0.5)
    vals = []
    last = None
    for _ in range(max(args.steps, 1)):
        last = cpu_baseline(cfg, wl, cfg["algorithm"], budget_s=budget)
        vals.append(last["value"])
    value = float(np.mean(vals))
    n_sample = last["positions"]
    line = {"metric": "positions/s fwd+adjoint", "value": value, "unit": "positions/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * n_sample / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": cfg["desc"], "sample_positions": n_sample},
            "cpu_baseline": {"value": value, "unit": "positions/s", "cores": last["cores"], "kind": "port",
                             "sample": last["sample"]},
            "e2e": {"value": value, "unit": "positions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="multislice", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--checkpoint", type=int, default=1,
                    help="256-px windows: keep every k-th slice's wave, recompute the rest")
    ap.add_argument("--no-optimizer", action="store_true",
                    help="skip the optimizer-step measurement (fourier_clean, L-BFGS epoch)")
    ap.add_argument("--train", type=int, default=2000, help="warm-start: training specimens")
    ap.add_argument("--test", type=int, default=100, help="warm-start: held-out specimens")
    ap.add_argument("--epochs", type=int, default=8, help="warm-start: training epochs")
    ap.add_argument("--recon-epochs", type=int, default=20, help="warm-start: L-BFGS epochs per reconstruction")
    ap.add_argument("--lr", type=float, default=1e-3, help="warm-start: Adam learning rate")
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config], name=args.config)
    if args.impl == "reference":
        return run_reference(args, cfg)
    if cfg.get("warm_start"):
        return run_warm_start(args, cfg)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)

    from pypty_gb300 import _lib
    from pypty_gb300.engine import Engine, Geometry, make_problem

    wl = build_workload(cfg)
    W, Z, Mp = cfg["W"], cfg["Z"], cfg["Mp"]
    eng = Engine(dev)
    geo = Geometry.make(wl["ipos"], wl["corr"])
    n_pos = geo.positions.shape[0]
    common = dict(algorithm=cfg["algorithm"], wavelength=wl["wavelength"], pixel_size_x=wl["px"],
                  pixel_size_y=wl["px"], slice_distance=wl["dz"], compute_batch=cfg["batch"])
    prob = make_problem(W, wl["obj0"].shape, Mp, geo, step_pos=True, checkpoint_every=args.checkpoint, **common)
    meas_d = simulate_measured(eng, prob, wl, geo)
    probe_d = torch.from_numpy(wl["probe"]).to(dev)
    obj_d = torch.from_numpy(wl["obj0"]).to(dev)
    out = (torch.empty(2, dtype=torch.float64, device=dev), torch.empty_like(obj_d), torch.empty_like(probe_d),
           torch.empty((n_pos, 2), dtype=torch.float32, device=dev))
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---------------- device-resident timing
    for _ in range(args.warmup):
        eng.loss_and_direction(prob, obj_d, probe_d, geo, meas_d, out=out)
    torch.cuda.synchronize(dev)
    barrier()
    torch.cuda.synchronize(dev)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n_batches = -(-n_pos // cfg["batch"])
    with ClockSampler(local_rank) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            eng.loss_and_direction(prob, obj_d, probe_d, geo, meas_d, out=out)
        stop.record(stream)
        torch.cuda.synchronize(dev)
    barrier()
    ms = start.elapsed_time(stop) / args.steps
    # the same steps again under the launch profiler: the library then issues every launch on
    # one stream, one after another, so each kernel's CUDA-event interval is that kernel alone
    # (the roofline's launch duration and the kernel shares)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with _lib.LaunchProfiler((16 + 12 * n_batches) * max(args.steps, 1)) as prof:
        p0.record(stream)
        for _ in range(args.steps):
            eng.loss_and_direction(prob, obj_d, probe_d, geo, meas_d, out=out)
        p1.record(stream)
        torch.cuda.synchronize(dev)
    profiled_ms = p0.elapsed_time(p1) / args.steps
    ms = max_over_ranks(ms, world, dev)
    loss_val = float(out[0][0].item())
    if not np.isfinite(loss_val):
        raise RuntimeError("non-finite loss in the benchmark")
    value = replica_throughput(n_pos, world, ms)

    # ---------------- end-to-end through the public call with host buffers
    obj_h = torch.from_numpy(wl["obj0"]).pin_memory()
    probe_h = torch.from_numpy(wl["probe"]).pin_memory()
    meas_h = meas_d.cpu().pin_memory()
    og_h = torch.empty_like(obj_h).pin_memory()
    pg_h = torch.empty_like(probe_h).pin_memory()
    posg_h = torch.empty((n_pos, 2), dtype=torch.float32).pin_memory()
    ls_h = torch.empty(2, dtype=torch.float64).pin_memory()
    obj_e, probe_e, meas_e = torch.empty_like(obj_d), torch.empty_like(probe_d), torch.empty_like(meas_d)

    def e2e_step():
        obj_e.copy_(obj_h, non_blocking=True)
        probe_e.copy_(probe_h, non_blocking=True)
        meas_e.copy_(meas_h, non_blocking=True)
        eng.loss_and_direction(prob, obj_e, probe_e, geo, meas_e, out=out)
        og_h.copy_(out[1], non_blocking=True)
        pg_h.copy_(out[2], non_blocking=True)
        posg_h.copy_(out[3], non_blocking=True)
        ls_h.copy_(out[0], non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize(dev)
    barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_ms = max_over_ranks(e2e_ms, world, dev)
    h2d = obj_h.numel() * 8 + probe_h.numel() * 8 + meas_h.numel() * 4 + geo.positions.nbytes + \
        geo.pos_correction.nbytes + geo.sequence.nbytes

    # ---------------- streamed patterns: the measured data stays in pinned host memory and the
    # kernels read it in place over the host link (datasets larger than HBM, load_one_by_one)
    for _ in range(args.warmup):
        eng.loss_and_direction(prob, obj_d, probe_d, geo, meas_h, out=out)
    torch.cuda.synchronize(dev)
    barrier()
    torch.cuda.synchronize(dev)
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(args.steps):
        eng.loss_and_direction(prob, obj_d, probe_d, geo, meas_h, out=out)
    s1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    streamed_ms = s0.elapsed_time(s1) / args.steps
    streamed_ms = max_over_ranks(streamed_ms, world, dev)
    d2h = og_h.numel() * 8 + pg_h.numel() * 8 + posg_h.numel() * 4 + 16

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---------------- roofline of the dominant kernel, timed live with CUDA events
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peaks = json.load(open(peaks_path))
        hbm_peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    else:
        hbm_peak, peak_src = 6800.0, "fallback"
    fused_ms = prof.ms.get("fused_multislice", 0.0)
    fused_n = max(prof.launches.get("fused_multislice", 0), 1)
    fused_avg_s = fused_ms / fused_n / 1000.0
    per_launch_pos = n_pos / (fused_n / args.steps)
    launch_bytes = alg_bytes_per_position(W, Z, Mp) * per_launch_pos
    achieved = launch_bytes / fused_avg_s / 1e9
    path_bytes = alg_bytes_per_position(W, Z, Mp) * n_pos
    total_prof_ms = sum(prof.ms.values())
    kernel_share = {k: round(v / total_prof_ms, 4) for k, v in sorted(prof.ms.items(), key=lambda kv: -kv[1])
                    if v > 0}
    cs = clocks.summary()
    line = {
        "metric": "positions/s fwd+adjoint", "value": value, "unit": "positions/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": cfg["desc"], "positions_per_step": n_pos, "global_batch": n_pos * world,
                   "checkpoint_every": args.checkpoint,
                   "workspace_gb": round(_lib.workspace_bytes(prob) / 1e9, 2),
                   "parallelism": "replicas x%d" % world if world > 1 else "single GPU",
                   "l2": "working set per step >> 129 MB L2 (inputs 110 MB + 2 GB wave stack per batch); no flush"},
        "e2e": {"value": replica_throughput(n_pos, world, e2e_ms), "unit": "positions/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "streamed_patterns": {"value": replica_throughput(n_pos, world, streamed_ms), "unit": "positions/s",
                              "ms_per_step": streamed_ms, "host_read_bytes_per_step": int(meas_h.numel() * 4),
                              "note": "measured patterns read in place from pinned host memory"},
        "roofline": {"bound": "hbm", "kernel": "fused_multislice", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "peak_source": peak_src + " (hbm_gbs)",
                     "traffic": (TRAFFIC_PER_POSITION[(W, Z, Mp)] * per_launch_pos
                                 if (W, Z, Mp) in TRAFFIC_PER_POSITION else None),
                     "traffic_source": "ncu dram bytes of a 64-position capture of the same shape, scaled by "
                                       "positions per launch (profiles/)",
                     "alg_bytes_per_launch": launch_bytes,
                     "alg_bytes_per_position": alg_bytes_per_position(W, Z, Mp),
                     "kernel_bytes_per_position": fused_bytes_per_position(W, Z, Mp),
                     "avg_launch_ms": fused_avg_s * 1e3,
                     "timing": "CUDA events around each launch in a second pass of the same steps with the "
                               "launch profiler on (launches serialised on one stream: kernels %.2f ms per step "
                               "there; %.2f ms per step in the timed region, where batches overlap on three "
                               "streams)" % (total_prof_ms / max(args.steps, 1), ms),
                     "profiled_pass_ms_per_step": profiled_ms},
        "path_roofline": {"alg_bytes_per_position": alg_bytes_per_position(W, Z, Mp),
                          "achieved_gbs": path_bytes / (ms / 1000.0) / 1e9,
                          "frac": path_bytes / (ms / 1000.0) / 1e9 / hbm_peak,
                          "fft_tflops": fft_flops_per_position(W, Z, Mp) * n_pos / (ms / 1000.0) / 1e12},
        "kernel_share": kernel_share,
        "gpu_launches": prof.total_launches,
        "clocks": {"sm_mhz": cs.get("sm_mhz"), "sm_max_mhz": cs.get("sm_max_mhz"), "reasons": cs.get("reasons")},
        "loss": loss_val,
    }
    if cfg.get("variants"):
        line["variants_path"] = variants_timing(eng, prob, geo, meas_d, obj_d, probe_d, n_pos)
    if cfg.get("sweep"):
        line["precision_sweep"] = precision_sweep(eng, wl, geo, meas_d, obj_d, probe_d, cfg, common,
                                                  n_sub=min(512, n_pos), batch=min(256, cfg["batch"]))
    if not args.no_optimizer:
        try:
            line["optimizer"] = optimizer_step(eng, prob, geo, meas_d, obj_d, probe_d, wl, ms, hbm_peak, peak_src)
        except (ValueError, RuntimeError) as exc:      # a diverging trial point: report, keep the line
            line["optimizer"] = {"error": str(exc)}
    if not args.no_cpu_baseline:
        cb = cpu_baseline(cfg, wl, cfg["algorithm"])
        one = cpu_baseline(cfg, wl, cfg["algorithm"], budget_s=10.0, cores=1)
        for d in (cb, one):
            d.pop("seconds", None)
            d.pop("positions", None)
        cb["one_core"] = {"value": one["value"], "unit": one["unit"], "cores": 1, "sample": one["sample"],
                          "note": "scipy.fft single-threaded, as the reference ships"}
        line["cpu_baseline"] = cb
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
