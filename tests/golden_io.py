"""Load the committed golden fixtures (reference outputs on seeded inputs)."""
import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def loss_case_names():
    names = []
    for p in sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))):
        n = os.path.basename(p)[:-4]
        if not n.startswith(("core_", "fourier_clean", "lbfgs_", "variant_")):
            names.append(n)
    return names


def load_case(name):
    d = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    s = d["scalars"]
    d.update(distance=float(s[0]), edge_mult=float(s[1]), wavelength=float(s[2]),
             px=float(s[3]), cutoff=float(s[4]), rolloff=float(s[5]),
             loss_weight=float(s[6]), batch=int(s[7]), step_probe=int(s[8]),
             step_obj=int(s[9]), step_pos=int(s[10]), algorithm=str(d["algorithm"]),
             double=bool(d["double"]))
    d.setdefault("distances", None)   # one distance per slice step, when the case has them
    return d


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def variant_case_names():
    return [os.path.basename(p)[len("variant_"):-4]
            for p in sorted(glob.glob(os.path.join(GOLDEN_DIR, "variant_*.npz")))]


def load_variant_case(name):
    """A near-field / compressed / beam-current / aberration fixture
    (``tests/golden/make_golden_variants.py``)."""
    d = dict(np.load(os.path.join(GOLDEN_DIR, "variant_" + name + ".npz")))
    s = d["scalars"]
    keys = ["distance", "edge_mult", "wavelength", "px", "cutoff", "rolloff", "loss_weight", "batch", "step_probe",
            "step_obj", "step_pos", "defocus", "cs", "alpha", "tan_x", "tan_y", "step_bc", "step_ab", "data_pad",
            "use_padded", "shift0", "shift1", "mult", "tilt_mode", "step_tilts", "upsample", "step_sb"]
    defaults = dict(upsample=1.0, step_sb=0.0)   # fixtures written before these scalars existed
    for i, k in enumerate(keys):
        d[k] = float(s[i]) if i < len(s) else defaults[k]
    for k in ("batch", "step_probe", "step_obj", "step_pos", "step_bc", "step_ab", "data_pad", "use_padded", "shift0",
              "shift1", "tilt_mode", "step_tilts", "upsample", "step_sb"):
        d[k] = int(d[k])
    d["algorithm"] = str(d["algorithm"])
    d["recon_type"] = str(d["recon_type"])
    d["double"] = bool(d["double"])
    for k in ("static_background", "ref_static_grad", "distances", "defocus_array", "probe_marker"):
        d.setdefault(k, np.zeros(0, np.float32))
    for k in ("masks", "beam_current", "aberrations", "aberration_marker", "tilts", "static_background", "distances",
              "defocus_array", "probe_marker"):
        if d[k].size == 0:
            d[k] = None
    return d
