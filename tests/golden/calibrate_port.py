"""Time the reference's own NumPy path against the oracle port on the same inputs.

The benchmark's CPU baseline runs the oracle (a NumPy restatement of the reference path,
``oracle/ptycho_oracle.py``) because the reference itself is not installed where the GPU
runs. This script measures how far the port's speed is from the reference's on the
benchmarked workload (128 px probe, 20 slices, 3 probe modes, Poisson loss, a 512^2 x 20
object, jittered 32 x 32 scan), on a fixed subset of positions, at one core (``scipy.fft``
single-threaded, as the reference ships: ``pypty/fft.py:111-156`` passes no ``workers``)
and with ``scipy.fft.set_workers(n)`` around both calls. It also checks that the two give
the same loss. Run where the reference checkout is available::

    PYPTY_REFERENCE_ROOT=<reference checkout> python tests/golden/calibrate_port.py [n_positions] [workers]

It prints one JSON line: positions/s of each at each core count and the ratio port /
reference.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import scipy.fft  # noqa: E402

import bench  # noqa: E402
from make_golden import ref_loss_and_direction  # noqa: E402
from oracle import ptycho_oracle as orc  # noqa: E402
from refimport import import_reference  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 16
    workers = int(sys.argv[2]) if len(sys.argv) > 2 else (os.cpu_count() or 1)
    pypty = import_reference()
    cfg = dict(bench.CONFIGS["multislice"], name="multislice")
    wl = bench.build_workload(cfg)
    rng = np.random.default_rng(5)
    seq = np.arange(n)
    meas = rng.poisson(50.0, (wl["ipos"].shape[0], cfg["W"], cfg["W"])).astype(np.float32)
    c = dict(double=False, positions=wl["ipos"], pos_correction=wl["corr"], distance=wl["dz"], edge_mult=1.0,
             measured=meas, algorithm=cfg["algorithm"], wavelength=wl["wavelength"], step_probe=1, step_obj=1,
             step_pos=1, px=wl["px"], cutoff=2 / 3, rolloff=0.0, sequence=seq, loss_weight=1, batch=cfg["batch"])

    def reference():
        return ref_loss_and_direction(pypty, c, wl["obj0"], wl["probe"])[0]

    def port():
        return orc.loss_and_direction(wl["obj0"], wl["probe"], wl["ipos"], wl["corr"], wl["dz"], 1.0, meas,
                                      cfg["algorithm"], wl["wavelength"], 1, 1, 1, wl["px"], wl["px"], 2 / 3, 0.0,
                                      seq, 1, cfg["batch"])[0]

    out = {"workload": cfg["desc"], "positions": n, "cpu_count": os.cpu_count()}
    for cores in (1, workers):
        row = {}
        with scipy.fft.set_workers(cores):
            for name, fn in (("reference", reference), ("port", port)):
                fn()                          # warm-up
                t0 = time.perf_counter()
                loss = fn()
                dt = time.perf_counter() - t0
                row[name] = {"positions_per_s": round(n / dt, 3), "seconds": round(dt, 2), "loss": float(loss)}
        row["port_over_reference"] = round(row["port"]["positions_per_s"] / row["reference"]["positions_per_s"], 3)
        row["loss_rel_diff"] = abs(row["port"]["loss"] - row["reference"]["loss"]) / abs(row["reference"]["loss"])
        out["cores_%d" % cores] = row
    print(json.dumps(out))


if __name__ == "__main__":
    main()
