"""GPU path against the reference (golden vectors) and the NumPy oracle.

Tolerances (complex64 path): loss relative error <= 1e-5, gradient relative L2 <= 1e-4
(object, probe and position gradients), FFTs relative L2 <= 2e-6 against float64 NumPy.
"""
import numpy as np
import pytest

from golden_io import load_case, loss_case_names, rel_l2

pytestmark = pytest.mark.gpu

LOSS_TOL = 1e-5
GRAD_TOL = 1e-4


@pytest.fixture(scope="module")
def engine():
    import torch
    from pypty_gb300.engine import Engine
    return Engine(torch.device("cuda", 0))


@pytest.mark.parametrize("W", [64, 128])
@pytest.mark.parametrize("inverse,shift", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_window_fft_matches_numpy(engine, W, inverse, shift):
    import torch
    rng = np.random.default_rng(W + 2 * inverse + shift)
    x = (rng.normal(size=(5, W, W)) + 1j * rng.normal(size=(5, W, W))).astype(np.complex64)
    out = engine.fft2(torch.from_numpy(x).cuda(), inverse=bool(inverse), shift=bool(shift)).cpu().numpy()
    xd = x.astype(np.complex128)
    if not inverse:
        ref = np.fft.fft2(xd, axes=(1, 2))
        ref = np.fft.fftshift(ref, axes=(1, 2)) if shift else ref
    else:
        ref = np.fft.ifft2(np.fft.ifftshift(xd, axes=(1, 2)) if shift else xd, axes=(1, 2))
    assert rel_l2(out, ref) <= 2e-6


def test_fft_mirror_over_reference_axes():
    from pypty_gb300 import fft as gfft
    rng = np.random.default_rng(3)
    x = (rng.normal(size=(3, 64, 64, 2, 1)) + 1j * rng.normal(size=(3, 64, 64, 2, 1))).astype(np.complex64)
    assert rel_l2(gfft.fft2(x, axes=(1, 2)), np.fft.fft2(x.astype(np.complex128), axes=(1, 2))) <= 2e-6
    y = np.fft.fftshift(np.fft.fft2(x.astype(np.complex128), axes=(1, 2)), axes=(1, 2))
    assert rel_l2(gfft.shift_fft2(x, axes=(1, 2)), y) <= 2e-6
    assert rel_l2(gfft.ifft2_ishift(y.astype(np.complex64), axes=(1, 2)), x) <= 2e-6


@pytest.mark.parametrize("name", loss_case_names())
def test_loss_and_direction_matches_reference(engine, name):
    from gpu_helpers import run_gpu
    c = load_case(name)
    loss, sse, og, pg, posg = run_gpu(c, engine=engine)
    assert abs(loss - float(c["ref_loss"])) <= LOSS_TOL * abs(float(c["ref_loss"]))
    assert abs(sse - float(c["ref_sse"])) <= LOSS_TOL * abs(float(c["ref_sse"]))
    assert rel_l2(og, c["ref_object_grad"]) <= GRAD_TOL
    if c["step_probe"]:
        assert rel_l2(pg, np.asarray(c["ref_probe_grad"]).reshape(pg.shape)) <= GRAD_TOL
    if c["step_pos"]:
        assert rel_l2(posg, c["ref_pos_grad"]) <= GRAD_TOL


def test_batch_size_does_not_change_result(engine):
    from gpu_helpers import run_gpu
    c = load_case("multislice_ml_c64")
    a = run_gpu(c, compute_batch=36, engine=engine)
    b = run_gpu(c, compute_batch=5, engine=engine)
    assert abs(a[0] - b[0]) <= 1e-9 * abs(a[0])
    assert rel_l2(b[2], a[2]) <= 1e-6 and rel_l2(b[3], a[3]) <= 1e-6 and rel_l2(b[4], a[4]) <= 1e-6


def test_results_are_bitwise_deterministic(engine):
    from gpu_helpers import run_gpu
    c = load_case("w128_modes_c64")
    a = run_gpu(c, engine=engine)
    b = run_gpu(c, engine=engine)
    assert a[0] == b[0] and a[1] == b[1]
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4])


def test_drop_in_objective_matches_reference():
    """The reference-signature mirror, called positionally like pypty/iterative.py:524."""
    from pypty_gb300 import objective
    c = load_case("modes_lsq_c64")
    f = np.float32
    tilts = np.zeros((1, 6), f)
    args = [c["obj"], c["probe"], c["positions"], c["pos_correction"], tilts, np.zeros_like(tilts),
            np.array([c["distance"]], f), c["edge_mult"], c["measured"], c["algorithm"], f(c["wavelength"]),
            c["step_probe"], c["step_obj"], c["step_pos"], 0, None, f(c["px"]), f(c["px"]), "far_field", 0,
            np.array([0.0]), 0, f(c["cutoff"]), f(c["rolloff"]), "multislice", c["sequence"], False, 1, 0,
            None, c["loss_weight"], 1, [0, 0], 1, None, 0, 0, None, None, None, c["batch"], False, None, 0, 0,
            f, np.complex64, np, True, None, 1, 0, 0, 0, 0, 0, 0, None, 0, 0, None, 0, 0, 0, 1, 2, 0, 0.5,
            0, 0, 0, 0.05, False, 0, False, False, True]
    res = objective.loss_and_direction(*args)
    assert len(res) == 10
    assert abs(res[0] - float(c["ref_loss"])) <= LOSS_TOL * abs(float(c["ref_loss"]))
    assert rel_l2(res[2], c["ref_object_grad"]) <= GRAD_TOL
    assert rel_l2(res[3], c["ref_probe_grad"]) <= GRAD_TOL
    assert rel_l2(res[4], c["ref_pos_grad"]) <= GRAD_TOL
    assert res[2].dtype == np.complex64 and res[2].shape == c["obj"].shape


def _oracle_case(W, Z, Mp, Mo, n_scan, algorithm, seed, batch, double=False):
    from oracle import ptycho_oracle as orc
    from pypty_gb300 import synth
    rng = np.random.default_rng(seed)
    px, kV = 0.1, 300.0
    n = W + int(n_scan * 7) + 8
    truth = synth.gaussian_phase_object(n, n, Z, 60, 0.3, px, 0.2, 1.0, rng, n_modes=Mo)
    probe = synth.make_probe(W, px, kV, 30.0, 50.0, Mp, 0.5 ** np.arange(Mp), 1e5)
    ipos, corr = synth.split_positions(synth.raster_positions(n_scan, n_scan, 7.0, 2.0, rng))
    lam = synth.wavelength_A(kV)
    seq = np.arange(ipos.shape[0])
    sim = orc.loss_and_direction(truth, probe, ipos, corr, 2.0, 1.0, None, algorithm, lam, 1, 1, 1, px, px,
                                 2 / 3, 0.0, seq, 1, batch, simulate=True)
    meas = synth.poisson_patterns(sim, 1.0, rng)
    obj0 = np.exp(0.6j * np.angle(truth)).astype(np.complex64)
    c = dict(obj=obj0, probe=probe, positions=ipos, pos_correction=corr, sequence=seq, measured=meas,
             algorithm=algorithm, wavelength=lam, px=px, cutoff=2 / 3, rolloff=0.0, distance=2.0,
             edge_mult=1.0, loss_weight=1, batch=batch, step_obj=1, step_probe=1, step_pos=1)
    f, cx = (np.float64, np.complex128) if double else (np.float32, np.complex64)
    ref = orc.loss_and_direction(obj0.astype(cx), probe.astype(cx), ipos, corr.astype(f), 2.0, 1.0,
                                 meas.astype(f), algorithm, lam, 1, 1, 1, px, px, 2 / 3, 0.0, seq, 1, batch,
                                 float_dtype=f, complex_dtype=cx)
    return c, ref


@pytest.mark.parametrize("W,Z,Mp,Mo,alg", [(128, 6, 3, 1, "ml"), (64, 5, 2, 2, "lsq_sqrt"),
                                           (128, 2, 8, 1, "lsq")])
def test_against_fp64_oracle(engine, W, Z, Mp, Mo, alg):
    """Larger shapes than the goldens (multislice, many modes) against the FP64 oracle."""
    from gpu_helpers import run_gpu
    c, ref = _oracle_case(W, Z, Mp, Mo, 3, alg, seed=W + Z + Mp, batch=4, double=True)
    loss, sse, og, pg, posg = run_gpu(c, engine=engine)
    assert abs(loss - ref[0]) <= LOSS_TOL * abs(ref[0])
    assert rel_l2(og, ref[2]) <= GRAD_TOL
    assert rel_l2(pg, ref[3]) <= GRAD_TOL
    assert rel_l2(posg, ref[4]) <= GRAD_TOL


def test_simulated_patterns_match_oracle(engine):
    import torch
    from oracle import ptycho_oracle as orc
    from pypty_gb300.engine import Geometry, make_problem
    c, _ = _oracle_case(64, 3, 2, 1, 3, "ml", seed=5, batch=4)
    sim_ref = orc.loss_and_direction(c["obj"], c["probe"], c["positions"], c["pos_correction"], 2.0, 1.0,
                                     None, "ml", c["wavelength"], 1, 1, 0, c["px"], c["px"], 2 / 3, 0.0,
                                     c["sequence"], 1, 4, float_dtype=np.float64,
                                     complex_dtype=np.complex128, simulate=True)
    geo = Geometry.make(c["positions"], c["pos_correction"], c["sequence"])
    prob = make_problem(64, c["obj"].shape, 2, geo, algorithm="ml", wavelength=c["wavelength"],
                        pixel_size_x=c["px"], pixel_size_y=c["px"], slice_distance=2.0, compute_batch=4)
    out = engine.simulate(prob, torch.from_numpy(c["obj"]).cuda(), torch.from_numpy(c["probe"]).cuda(), geo)
    assert rel_l2(out.cpu().numpy(), sim_ref) <= 2e-6


def test_simulated_patterns_do_not_depend_on_batching(engine):
    """Patterns are per position: one batch and eight double-buffered batches on two streams
    give the same bits."""
    import torch
    from pypty_gb300.engine import Geometry, make_problem
    c = load_case("w128_modes_c64")
    dev = torch.device("cuda", 0)
    obj = torch.from_numpy(np.ascontiguousarray(c["obj"]).astype(np.complex64)).to(dev)
    probe = torch.from_numpy(np.ascontiguousarray(c["probe"]).astype(np.complex64)).to(dev)
    geo = Geometry.make(c["positions"], c["pos_correction"], c["sequence"])
    outs = []
    for batch in (len(c["sequence"]), 1):
        prob = make_problem(probe.shape[0], tuple(obj.shape), probe.shape[2], geo, algorithm=c["algorithm"],
                            wavelength=float(np.float32(c["wavelength"])), pixel_size_x=float(np.float32(c["px"])),
                            pixel_size_y=float(np.float32(c["px"])), slice_distance=c["distance"],
                            edge_mult=c["edge_mult"], compute_batch=batch)
        outs.append(engine.simulate(prob, obj, probe, geo).cpu().numpy())
    assert np.array_equal(outs[0], outs[1])


def test_drop_in_objective_with_per_slice_distances():
    """this_distances with one entry per slice step through the reference-signature mirror."""
    from pypty_gb300 import objective
    from test_host_logic import base_kwargs
    c = load_case("distances_ml_c64")
    f = np.float32
    kw = base_kwargs(this_obj=c["obj"], full_probe=c["probe"], this_pos_array=c["positions"],
                     this_pos_correction=c["pos_correction"], this_distances=np.asarray(c["distances"], f),
                     edge_slice_thickness_multiplier=c["edge_mult"], measured_array=c["measured"],
                     algorithm_type=c["algorithm"], this_wavelength=f(c["wavelength"]),
                     this_step_probe=c["step_probe"], this_step_obj=c["step_obj"],
                     this_step_pos_correction=c["step_pos"], pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]),
                     damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(c["rolloff"]),
                     this_chopped_sequence=c["sequence"], this_loss_weight=c["loss_weight"],
                     compute_batch=c["batch"])
    res = objective.loss_and_direction(**kw)
    assert abs(res[0] - float(c["ref_loss"])) <= LOSS_TOL * abs(float(c["ref_loss"]))
    assert rel_l2(res[2], c["ref_object_grad"]) <= GRAD_TOL
    assert rel_l2(res[3], c["ref_probe_grad"]) <= GRAD_TOL
    assert rel_l2(res[4], c["ref_pos_grad"]) <= GRAD_TOL


def test_drop_in_saves_simulated_patterns(tmp_path):
    """data_simulation_flag: the mean-over-modes model patterns of every position are saved
    (float64, detector order) while the loss and gradients are returned as usual."""
    from oracle import ptycho_oracle as orc
    from pypty_gb300 import objective
    from test_host_logic import base_kwargs
    c = load_case("multislice_ml_c64")
    f = np.float32
    path = str(tmp_path / "sim.npy")
    kw = base_kwargs(this_obj=c["obj"], full_probe=c["probe"], this_pos_array=c["positions"],
                     this_pos_correction=c["pos_correction"], this_distances=np.array([c["distance"]], f),
                     edge_slice_thickness_multiplier=c["edge_mult"], measured_array=c["measured"],
                     algorithm_type=c["algorithm"], this_wavelength=f(c["wavelength"]),
                     this_step_probe=c["step_probe"], this_step_obj=c["step_obj"],
                     this_step_pos_correction=c["step_pos"], pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]),
                     damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(c["rolloff"]),
                     this_chopped_sequence=c["sequence"], this_loss_weight=c["loss_weight"],
                     compute_batch=c["batch"], data_simulation_flag=path)
    res = objective.loss_and_direction(**kw)
    assert abs(res[0] - float(c["ref_loss"])) <= LOSS_TOL * abs(float(c["ref_loss"]))
    sim = np.load(path)
    ref = orc.loss_and_direction(c["obj"].astype(np.complex128), c["probe"].astype(np.complex128), c["positions"],
                                 c["pos_correction"].astype(np.float64), c["distance"], c["edge_mult"], None,
                                 c["algorithm"], c["wavelength"], 1, 1, 0, c["px"], c["px"], c["cutoff"],
                                 c["rolloff"], c["sequence"], 1, c["batch"], float_dtype=np.float64,
                                 complex_dtype=np.complex128, simulate=True)
    assert sim.dtype == np.float64 and sim.shape == ref.shape
    assert rel_l2(sim, ref) <= 1e-5


def test_empty_sequence_gives_zero_loss_and_gradients():
    """No positions in the sequence: the reference's batch loop does not run, so the loss, sse
    and every gradient are zero (pypty/objective.py:372-382)."""
    from pypty_gb300 import objective
    from test_host_logic import base_kwargs
    c = load_case("multislice_ml_c64")
    f = np.float32
    kw = base_kwargs(this_obj=c["obj"], full_probe=c["probe"], this_pos_array=c["positions"],
                     this_pos_correction=c["pos_correction"], this_distances=np.array([c["distance"]], f),
                     measured_array=c["measured"], algorithm_type=c["algorithm"], this_wavelength=f(c["wavelength"]),
                     this_step_pos_correction=1, pixel_size_x_A=f(c["px"]), pixel_size_y_A=f(c["px"]),
                     this_chopped_sequence=np.zeros(0, np.int64), compute_batch=c["batch"])
    res = objective.loss_and_direction(**kw)
    assert res[0] == 0.0 and res[1] == 0.0
    assert not np.any(res[2]) and not np.any(res[3]) and not np.any(res[4])
    assert res[2].shape == c["obj"].shape and res[4].shape == c["pos_correction"].shape


@pytest.mark.parametrize("W", [64, 128, 256])
def test_windows_at_object_edges(engine, W):
    """Windows that touch every edge of a non-square object (first and last valid row and
    column), in a ragged last batch, against the FP64 oracle."""
    from gpu_helpers import run_gpu
    from oracle import ptycho_oracle as orc
    from pypty_gb300 import synth
    rng = np.random.default_rng(W + 11)
    px, kV, Z, Mp = 0.1, 300.0, 3, 2
    ny, nx = W + 20, W + 37
    truth = synth.gaussian_phase_object(ny, nx, Z, 40, 0.3, px, 0.2, 1.0, rng)
    probe = synth.make_probe(W, px, kV, 30.0, 50.0, Mp, 0.5 ** np.arange(Mp), 1e5)
    ipos = np.array([[0, 0], [0, nx - W], [ny - W, 0], [ny - W, nx - W], [7, 13]], np.int32)
    corr = rng.uniform(-0.5, 0.5, ipos.shape).astype(np.float32)
    seq = np.array([3, 0, 4, 1, 2])
    lam = synth.wavelength_A(kV)
    sim = orc.loss_and_direction(truth, probe, ipos, corr, 2.0, 1.0, None, "ml", lam, 1, 1, 1, px, px,
                                 2 / 3, 0.0, seq, 1, 2, simulate=True)
    meas = synth.poisson_patterns(sim, 1.0, rng)
    obj0 = np.exp(0.6j * np.angle(truth)).astype(np.complex64)
    c = dict(obj=obj0, probe=probe, positions=ipos, pos_correction=corr, sequence=seq, measured=meas,
             algorithm="ml", wavelength=lam, px=px, cutoff=2 / 3, rolloff=0.0, distance=2.0,
             edge_mult=1.0, loss_weight=1, batch=2, step_obj=1, step_probe=1, step_pos=1)
    ref = orc.loss_and_direction(obj0.astype(np.complex128), probe.astype(np.complex128), ipos,
                                 corr.astype(np.float64), 2.0, 1.0, meas.astype(np.float64), "ml", lam,
                                 1, 1, 1, px, px, 2 / 3, 0.0, seq, 1, 2, float_dtype=np.float64,
                                 complex_dtype=np.complex128)
    # the same computation in complex64 on the CPU: its distance from FP64 is the floor that
    # single precision sets for these inputs (at 256 px about 1e-4 for the object and probe
    # gradients); the GPU result stays within 1e-4 or three times that floor
    r32 = orc.loss_and_direction(obj0, probe.astype(np.complex64), ipos, corr, 2.0, 1.0, meas.astype(np.float32),
                                 "ml", lam, 1, 1, 1, px, px, 2 / 3, 0.0, seq, 1, 2, float_dtype=np.float32,
                                 complex_dtype=np.complex64)
    loss, sse, og, pg, posg = run_gpu(c, engine=engine)
    assert abs(loss - ref[0]) <= LOSS_TOL * abs(ref[0])
    for k, g in ((2, og), (3, pg), (4, posg)):
        assert rel_l2(g, ref[k]) <= max(GRAD_TOL, 3 * rel_l2(r32[k], ref[k])), (k, rel_l2(g, ref[k]))
    # the object gradient reaches the last row and column
    assert np.abs(og[-1]).max() > 0 and np.abs(og[:, -1]).max() > 0


def test_pinned_patterns_follow_in_place_changes():
    """With load_one_by_one the patterns are read from a pinned host buffer; the reference
    reads the caller's array on every call (objective.py:398-409), so a change made in place
    between two calls must reach the kernels."""
    import torch
    from pypty_gb300 import objective
    meas = np.ones((3, 64, 64), np.float32)
    a = objective.measured_tensor(meas, torch.device("cuda", 0), True)
    assert a.is_pinned() and float(a[1, 2, 3]) == 1.0
    meas[1, 2, 3] = 7.0
    b = objective.measured_tensor(meas, torch.device("cuda", 0), True)
    assert float(b[1, 2, 3]) == 7.0
