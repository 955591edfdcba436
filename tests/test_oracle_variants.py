"""Pin the variants oracle (near field, compressed detectors, beam current, aberration plates,
tilts, measured-data preprocessing, detector upsampling, static background) to golden vectors
produced by the reference's own NumPy path."""
import numpy as np
import pytest

from golden_io import load_variant_case, rel_l2, variant_case_names
from oracle import variants_oracle as vor


def run_variant_oracle(c):
    f, cx = (np.float64, np.complex128) if c["double"] else (np.float32, np.complex64)
    return vor.loss_and_direction_variants(
        c["obj"], c["probe"], c["positions"], c["pos_correction"],
        c["distance"] if c["distances"] is None else c["distances"], c["edge_mult"], c["measured"],
        c["algorithm"], c["wavelength"], c["step_probe"], c["step_obj"], c["step_pos"], c["px"], c["px"],
        c["cutoff"], c["rolloff"], c["sequence"], c["loss_weight"], c["batch"], recon_type=c["recon_type"],
        defocus=c["defocus"] if c["defocus_array"] is None else c["defocus_array"], cs=c["cs"],
        alpha_near_field=c["alpha"], tan_x=c["tan_x"], tan_y=c["tan_y"],
        masks=c["masks"], beam_current=c["beam_current"], step_beam_current=c["step_bc"],
        aberrations=c["aberrations"], aberration_marker=c["aberration_marker"], step_aberrations=c["step_ab"],
        data_pad=c["data_pad"], use_padded_intensity=c["use_padded"], data_shift_vector=(c["shift0"], c["shift1"]),
        data_multiplier=f(c["mult"]), tilts=c["tilts"], tilt_mode=c["tilt_mode"], step_tilts=c["step_tilts"],
        upsample_pattern=c["upsample"], static_background=c["static_background"],
        step_static_background=c["step_sb"], probe_marker=c["probe_marker"], float_dtype=f, complex_dtype=cx)


@pytest.mark.parametrize("name", variant_case_names())
def test_variants_oracle_matches_reference(name):
    c = load_variant_case(name)
    loss, sse, og, pg, posg, bcg, abg, tg, sbg = run_variant_oracle(c)
    tol = 1e-12 if c["double"] else 5e-6
    assert abs(float(loss) - float(c["ref_loss"])) <= tol * abs(float(c["ref_loss"]))
    assert abs(float(sse) - float(c["ref_sse"])) <= tol * abs(float(c["ref_sse"]))
    assert rel_l2(og, c["ref_object_grad"]) <= tol
    if c["step_probe"]:
        assert rel_l2(pg, np.asarray(c["ref_probe_grad"]).reshape(pg.shape)) <= tol
    if c["step_pos"]:
        assert rel_l2(posg, c["ref_pos_grad"]) <= (1e-12 if c["double"] else 1e-5)
    if c["step_bc"]:
        assert rel_l2(bcg, c["ref_beam_current_grad"]) <= (1e-12 if c["double"] else 1e-5)
    if c["step_ab"]:
        assert rel_l2(abg, c["ref_aberrations_grad"]) <= (1e-12 if c["double"] else 1e-5)
    if c["step_tilts"]:
        assert rel_l2(tg, c["ref_tilts_grad"]) <= (1e-12 if c["double"] else 1e-5)
    if c["step_sb"]:
        assert rel_l2(sbg, c["ref_static_grad"]) <= (1e-12 if c["double"] else 1e-5)


def test_near_field_alpha_is_rejected():
    """The reference's partial-coherence branch raises; the oracle refuses it too."""
    c = load_variant_case("near_c64")
    c = dict(c, alpha=1e-3)
    with pytest.raises(ValueError):
        run_variant_oracle(c)


def test_aberration_basis_order():
    """Krivanek order of the aberration basis (utils.py:1272-1308): C10, C12a, C12b, C21a, C21b,
    C23a, C23b, C30, ..."""
    n, m, ab = vor.convert_num_to_nmab(8)
    assert n == [1, 1, 1, 2, 2, 2, 2, 3]
    assert m == [0, 2, 2, 1, 1, 3, 3, 0]
    assert ab == ["", "a", "b", "a", "b", "a", "b", ""]


def test_single_tilt_inside_gradient_with_batches_raises_like_the_reference():
    """One tilt row, inside-tilt refinement and several positions per batch: the reference adds
    a (B,) vector into one row (multislice_core.py:180-182) and raises; so does the oracle."""
    c = load_variant_case("tilt0_single_c64")
    c = dict(c, batch=3)
    with pytest.raises(ValueError):
        run_variant_oracle(c)
