"""multislice / multislice_grads / scatteradd drop-ins against the reference's own outputs
(tests/golden/core_multislice_c64.npz) and against np.add.at."""
import numpy as np
import pytest

from golden_io import GOLDEN_DIR, rel_l2

pytestmark = pytest.mark.gpu


def _core():
    import os
    return dict(np.load(os.path.join(GOLDEN_DIR, "core_multislice_c64.npz")))


def test_multislice_matches_reference():
    from pypty_gb300 import multislice_core as mc
    d = _core()
    B, W, _, Z, Mo = d["obj_b"].shape
    Mp = d["probe_b"].shape[-1]
    waves = np.zeros((B, W, W, Z, Mp, Mo, 1), np.complex64)
    prop = d["prop"][None, :, :, None, None]
    waves, exit_w = mc.multislice(d["probe_b"], d["obj_b"], Z, Mo, Mp, np.array([1.5], np.float32),
                                  float(d["edge_mult"]), None, None, None, None, None, True, 0, 0, 2 / 3, 0, prop,
                                  None, d["mask"][None], waves, None, 0, 0, np.float32, np.complex64)
    assert rel_l2(waves[..., 0], d["ref_stack"]) <= 1e-5
    assert rel_l2(exit_w, d["ref_exit"]) <= 1e-5


def test_multislice_grads_matches_reference():
    from pypty_gb300 import multislice_core as mc
    d = _core()
    B, W, _, Z, Mo = d["obj_b"].shape
    Mp = d["probe_b"].shape[-1]
    pos = d["positions"]
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    my = pos[:, 0][:, None, None] + runy[None]
    mx = pos[:, 1][:, None, None] + runx[None]
    og = np.zeros_like(d["ref_object_grad"])
    prop = d["prop"][None, :, :, None, None]
    og, pgrad, _ = mc.multislice_grads(d["g_out"].copy(), d["ref_stack"][..., None].copy(), d["obj_b"], og, None,
                                       True, np.array([1.5], np.float32), float(d["edge_mult"]), None, None, None,
                                       None, 0, None, 0, Z, Mo, 0, prop, 0, 2 / 3, 0, 0, B, d["mask"][None], 1, 1,
                                       0, my, mx, np.float32, np.complex64, True)
    assert rel_l2(og, d["ref_object_grad"]) <= 1e-4
    assert rel_l2(pgrad, d["ref_probe_grad"]) <= 1e-4


def test_scatteradd_matches_add_at_and_accumulates():
    from pypty_gb300 import multislice_core as mc
    rng = np.random.default_rng(8)
    W, B, Ny, Nx, K = 64, 7, 150, 170, 3
    pos = np.stack([rng.integers(0, Ny - W, B), rng.integers(0, Nx - W, B)], 1)
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    my = pos[:, 0][:, None, None] + runy[None]
    mx = pos[:, 1][:, None, None] + runx[None]
    chop = (rng.normal(size=(B, W, W, K)) + 1j * rng.normal(size=(B, W, W, K))).astype(np.complex64)
    full = (rng.normal(size=(Ny, Nx, K)) + 1j * rng.normal(size=(Ny, Nx, K))).astype(np.complex64)
    ref = full.astype(np.complex128)
    np.add.at(ref, (my, mx), chop.astype(np.complex128))
    mc.scatteradd(full, my, mx, chop)
    assert rel_l2(full, ref) <= 1e-6
