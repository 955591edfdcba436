"""Pin the NumPy oracle to golden vectors produced by the reference's own NumPy path."""
import numpy as np
import pytest

from golden_io import load_case, loss_case_names, rel_l2
from oracle import ptycho_oracle as orc


def run_oracle(c):
    f, cx = (np.float64, np.complex128) if c["double"] else (np.float32, np.complex64)
    return orc.loss_and_direction(
        c["obj"], c["probe"], c["positions"], c["pos_correction"],
        c["distance"] if c["distances"] is None else c["distances"],
        c["edge_mult"], c["measured"], c["algorithm"], c["wavelength"], c["step_probe"],
        c["step_obj"], c["step_pos"], c["px"], c["px"], c["cutoff"], c["rolloff"],
        c["sequence"], c["loss_weight"], c["batch"], float_dtype=f, complex_dtype=cx)


@pytest.mark.parametrize("name", loss_case_names())
def test_oracle_matches_reference(name):
    c = load_case(name)
    loss, sse, og, pg, posg = run_oracle(c)
    # complex128 agrees to 1e-12 (same algorithm); complex64 differs only by pocketfft
    # rounding between the strided views the reference transforms and contiguous copies.
    tol = 1e-12 if c["double"] else 5e-6
    assert abs(float(loss) - float(c["ref_loss"])) <= tol * abs(float(c["ref_loss"]))
    assert abs(float(sse) - float(c["ref_sse"])) <= tol * abs(float(c["ref_sse"]))
    assert rel_l2(og, c["ref_object_grad"]) <= tol
    if c["step_probe"]:
        assert rel_l2(pg, np.asarray(c["ref_probe_grad"]).reshape(pg.shape)) <= tol
    if c["step_pos"]:
        assert rel_l2(posg, c["ref_pos_grad"]) <= (1e-12 if c["double"] else 1e-5)  # float32 sums, other order


def test_core_multislice_matches_reference():
    d = dict(np.load("tests/golden/core_multislice_c64.npz"))
    stack, exit_w = orc.multislice(d["probe_b"], d["obj_b"], d["prop"], float(d["edge_mult"]))
    assert rel_l2(stack, d["ref_stack"]) <= 1e-6
    assert rel_l2(exit_w, d["ref_exit"]) <= 1e-6
    grad_w, pgrad = orc.multislice_grads(d["g_out"], stack, d["obj_b"], d["prop"],
                                         float(d["edge_mult"]), d["mask"])
    W = d["probe_b"].shape[1]
    og = np.zeros_like(d["ref_object_grad"])
    pos = d["positions"]
    runx, runy = np.meshgrid(np.arange(W), np.arange(W), indexing="xy")
    orc.scatteradd(og, pos[:, 0][:, None, None] + runy[None], pos[:, 1][:, None, None] + runx[None],
                   grad_w)
    assert rel_l2(og, d["ref_object_grad"]) <= 1e-6
    assert rel_l2(pgrad, d["ref_probe_grad"]) <= 1e-6


def test_fp64_oracle_bounds_fp32_reference():
    """The complex64 reference result sits within the stated tolerance of the FP64 one."""
    for base in ["single_slice", "multislice_ml"]:
        c32 = load_case(base + "_c64")
        c64 = load_case(base + "_c128")
        assert abs(float(c32["ref_loss"]) - float(c64["ref_loss"])) <= 1e-5 * abs(float(c64["ref_loss"]))
        assert rel_l2(c32["ref_object_grad"], c64["ref_object_grad"]) <= 1e-4
