"""GPU optimizer step against the reference's outputs and the NumPy oracle.

* fourier_clean (``pty_fourier_clean``): relative L2 <= 1e-5 against the reference's /
  the oracle's complex64 result (FP32 FFTs against pocketfft), bitwise repeatable.
* L-BFGS vector algebra (``pty_lbfgs_*``): the two-loop direction against an FP64 NumPy
  two-loop on random pairs, relative L2 <= 1e-5.
* ``bfgs_update`` with the reference signature, several calls from an empty history:
  the same line-search decisions (trial count, accepted step) as the reference, loss
  relative error <= 1e-4, arrays relative L2 <= 1e-3 after every call.
"""
import os
import sys
import types

import numpy as np
import pytest

from golden_io import rel_l2
from oracle import lbfgs_oracle as lo
from test_oracle_lbfgs import LBFGS_CASES, load_lbfgs

pytestmark = pytest.mark.gpu

CLEAN_TOL = 1e-5


def _cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_fourier_clean_matches_reference_golden():
    from pypty_gb300 import utils
    d = dict(np.load("tests/golden/fourier_clean_c64.npz"))
    for name in ["a2", "a3", "a4", "a4r"]:
        cut, roll = d[name + "_cut"]
        res = utils.fourier_clean(d[name + "_in"], cutoff=np.float32(cut), rolloff=np.float32(roll))
        assert res.dtype == np.complex64
        assert rel_l2(res, d[name + "_out"]) <= CLEAN_TOL, name
    res = utils.fourier_clean(d["m_in"], mask=d["m_mask"])
    assert rel_l2(res, d["m_out"]) <= CLEAN_TOL


@pytest.mark.parametrize("shape,cut,roll", [
    ((512, 512, 20, 1), 2 / 3 - 0.005, 0.0),      # the 512^2 x 20 benchmark object
    ((256, 1024, 3, 1), 0.6, 0.15),                # non-square, roll-off
    ((2048, 2048, 2, 1), 2 / 3 - 0.005, 0.0),      # the largest benchmark extent
    ((4096, 64, 1, 1), 0.5, 0.0),                  # 1D-like, one plane
    ((128, 128, 5, 3), 0.7, 0.05),                 # odd plane count
])
def test_fourier_clean_matches_oracle(shape, cut, roll):
    import torch
    from pypty_gb300.optim import fourier_clean_
    rng = np.random.default_rng(sum(shape))
    x = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)
    dx = (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)
    c, r = np.float32(cut), np.float32(roll)
    xd, dxd = _cuda(x), _cuda(dx)
    out = fourier_clean_(xd, c, r)
    ref = lo.fourier_clean(x, cutoff=c, rolloff=r)
    assert rel_l2(out.cpu().numpy(), ref) <= CLEAN_TOL
    # the trial point x + step dx in the same first pass
    step = np.float32(0.37)
    out2 = fourier_clean_(xd, c, r, dx=dxd, step=float(step))
    ref2 = lo.fourier_clean(x + step * dx, cutoff=c, rolloff=r)
    assert rel_l2(out2.cpu().numpy(), ref2) <= CLEAN_TOL
    # in place, and bitwise repeatable
    y = xd.clone()
    fourier_clean_(y, c, r, out=y)
    torch.cuda.synchronize()
    assert torch.equal(y, out)


def test_fourier_clean_is_a_projection_for_a_hard_mask():
    from pypty_gb300.optim import fourier_clean_
    rng = np.random.default_rng(3)
    x = (rng.normal(size=(256, 256, 4)) + 1j * rng.normal(size=(256, 256, 4))).astype(np.complex64)
    a = fourier_clean_(_cuda(x), np.float32(0.6), 0.0)
    b = fourier_clean_(a, np.float32(0.6), 0.0)
    assert rel_l2(b.cpu().numpy(), a.cpu().numpy()) <= 2e-6


def test_unsupported_extent_raises():
    from pypty_gb300 import _lib
    from pypty_gb300.optim import fourier_clean_
    x = _cuda(np.zeros((96, 128, 1), np.complex64))
    with pytest.raises(_lib.PtyError):
        fourier_clean_(x, 0.6, 0.0)


def _two_loop_numpy(g, S, Y, w):
    """FP64 L-BFGS two-loop with per-segment gammas of the last pair
    (pypty/iterative.py:583-681, weights w per segment)."""
    def dot(a, b):
        return sum(wi * np.dot(ai.astype(np.float64), bi.astype(np.float64)) for wi, ai, bi in zip(w, a, b))
    rho = [1.0 / dot(y, s) for s, y in zip(S, Y)]
    q = [x.astype(np.float64).copy() for x in g]
    al = [0.0] * len(S)
    for i in range(len(S) - 1, -1, -1):
        al[i] = rho[i] * dot(S[i], q)
        q = [qi - al[i] * yi for qi, yi in zip(q, Y[i])]
    gam = [wi * np.dot(Y[-1][k].astype(np.float64), S[-1][k]) / np.dot(Y[-1][k].astype(np.float64), Y[-1][k])
           for k, wi in enumerate(w)]
    q = [qi * gk for qi, gk in zip(q, gam)]
    for i in range(len(S)):
        beta = al[i] - rho[i] * dot(Y[i], q)
        q = [qi + beta * si for qi, si in zip(q, S[i])]
    return [-qi for qi in q]


@pytest.mark.parametrize("nseg", [3, 7])
def test_two_loop_matches_fp64_numpy(nseg):
    import ctypes
    import torch
    from pypty_gb300 import _lib
    from pypty_gb300.optim import _ptrs
    rng = np.random.default_rng(7)
    # object, probe, positions (floats); then tilt rows, static background, aberrations, beam
    # currents
    sizes = [2 * 64 * 64 * 3, 2 * 32 * 32 * 2, 2 * 50, 6 * 50, 32 * 32, 2 * 7, 50][:nseg]
    w = [2.0, 2.0, 1.0, 1.0, 1.0, 1.0, 1.0][:nseg]
    m = 4
    g = [rng.normal(size=n).astype(np.float32) for n in sizes]
    # pairs with positive curvature y.s > 0, as accepted Wolfe steps give
    S, Y = [], []
    for _ in range(m):
        s = [rng.normal(size=n).astype(np.float32) for n in sizes]
        y = [(0.5 * si + 0.1 * rng.normal(size=si.size)).astype(np.float32) for si in s]
        S.append(s)
        Y.append(y)
    lib = _lib.lib()
    vs = _lib.VSpace()
    vs.n_seg, vs.obj_seg = nseg, 0
    for i in range(nseg):
        vs.n[i], vs.weight[i] = sizes[i], w[i]
    n = ctypes.c_size_t(0)
    lib.pty_lbfgs_state_bytes(ctypes.byref(n))
    state = torch.empty(n.value, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.pty_lbfgs_reset(ctypes.byref(vs), state.data_ptr(), st), "reset")
    gd = [_cuda(x) for x in g]
    qd = [torch.empty_like(x) for x in gd]
    Sd = [[_cuda(x) for x in s] for s in S]
    Yd = [[_cuda(x) for x in y] for y in Y]
    # push the pairs through pty_lbfgs_accept (step 1, dir = s, new_grad = g + y) to set rho / gamma
    for i in range(m):
        ng = [a + b for a, b in zip(gd, Yd[i])]
        s_out = [torch.empty_like(x) for x in gd]
        y_out = [torch.empty_like(x) for x in gd]
        _lib.check(lib.pty_lbfgs_accept(ctypes.byref(vs), 1.0, _ptrs(Sd[i]), _ptrs(gd), _ptrs(ng), _ptrs(s_out),
                                        _ptrs(y_out), i, state.data_ptr(), st), "accept")
        Sd[i], Yd[i] = s_out, y_out
    slots = (ctypes.c_int32 * m)(*range(m))
    _lib.check(lib.pty_lbfgs_two_loop(ctypes.byref(vs), _ptrs(gd), _ptrs(qd), m,
                                      _ptrs([t for s in Sd for t in s]), _ptrs([t for y in Yd for t in y]), slots,
                                      state.data_ptr(), st), "two_loop")
    ref = _two_loop_numpy(g, [[t.cpu().numpy() for t in s] for s in Sd], [[t.cpu().numpy() for t in y] for y in Yd],
                          w)
    got = np.concatenate([t.cpu().numpy() for t in qd])
    assert rel_l2(got, np.concatenate(ref)) <= 1e-5
    # d_value = <q, g>, weighted, FP64
    _lib.check(lib.pty_lbfgs_dot(ctypes.byref(vs), _ptrs(qd), _ptrs(gd), 0, state.data_ptr(), st), "dot")
    out = (ctypes.c_double * (2 + 2 * _lib.VSPACE_MAX_SEG))()
    _lib.check(lib.pty_lbfgs_read(state.data_ptr(), out, st), "read")
    dv = sum(wi * np.dot(qi.astype(np.float64), gi) for wi, qi, gi in
             zip(w, [t.cpu().numpy() for t in qd], g))
    assert out[0] == pytest.approx(dv, rel=1e-9)


def test_orthogonalize_modes_matches_oracle():
    from pypty_gb300.optim import orthogonalize_modes_
    rng = np.random.default_rng(9)
    p = (rng.normal(size=(64, 64, 4)) + 1j * rng.normal(size=(64, 64, 4))).astype(np.complex64)
    got = orthogonalize_modes_(_cuda(p.copy())).cpu().numpy()
    assert rel_l2(got, lo.make_states_orthogonal(p)) <= 1e-5


def _fake_reference_module(c):
    """A module holding the reference's iterative-module variables (pypty/iterative.py)."""
    ns = types.ModuleType("fake_iterative")
    ns.obj, ns.probe = c["obj"].copy(), c["probe"].copy()
    ns.positions, ns.positions_correction = c["positions"].copy(), c["corr"].copy()
    ns.tilts = np.zeros((1, 6), np.float32)
    ns.tilts_correction = np.zeros((1, 6), np.float32)
    ns.static_background = ns.aberrations_array = ns.beam_current = None
    ns.history_bfgs = None
    return ns


def _call(fn, c, epoch, warnings, failed):
    f, cx = np.float32, np.complex64
    return fn(
        algorithm_type=c["algorithm"], this_slice_distances=np.array([c["distance"]], dtype=f),
        edge_slice_thickness_multiplier=c["edge_mult"], this_step_probe=int(c["step_probe"]),
        this_step_obj=int(c["step_obj"]), this_step_pos_correction=int(c["step_pos"]), this_step_tilts=0,
        measured_array=c["measured"], this_wavelength=f(c["wavelength"]), masks=None, pixel_size_x_A=f(c["px"]),
        pixel_size_y_A=f(c["px"]), phase_norm_weight=0, abs_norm_weight=0, stepsize_threshold_low=1e-20,
        probe_reg_weight=0, aperture_mask=None, recon_type="far_field", defocus_array=np.array([0.0], dtype=f),
        Cs=f(0), alpha_near_field=f(0), damping_cutoff_multislice=f(c["cutoff"]), smooth_rolloff=f(c["rolloff"]),
        update_extra_cut=f(0.005), keep_probe_states_orthogonal=c["orthogonal"], do_charge_flip=False,
        cf_delta_phase=0, cf_delta_abs=0, cf_beta_phase=0, cf_beta_abs=0, phase_only_obj=False, wedge_mu=0,
        beta_wedge=0, wolfe_c1_constant=0.1, wolfe_c2_constant=0.9, atv_weight=0, atv_q=1, atv_p=2,
        tune_only_probe_phase=False, propmethod="multislice", this_chopped_sequence=c["sequence"],
        load_one_by_one=False, data_multiplier=f(1), data_pad=0, phase_plate_in_h5=None, print_flag=0,
        this_loss_weight=c["loss_weight"], max_count=20, reduce_factor=f(0.1), optimism=3, mixed_variance_weight=0,
        mixed_variance_sigma=0.5, data_bin=1, data_shift_vector=[0, 0], smart_memory=False, default_float=f,
        default_complex=cx, default_int=np.int32, upsample_pattern=1, this_step_static_background=0, tilt_mode=0,
        fancy_sigma=None, tune_only_probe_abs=False, aberration_marker=None, this_step_aberrations_array=0,
        probe_marker=None, compute_batch=c["batch"], current_window=None, current_window_weight=0,
        dynamically_resize_yx_object=False, lazy_clean=c["lazy_clean"], current_gaussian_filter=False,
        current_apply_gaussian_filter_amplitude=False, this_beam_current_step=0, xp=np, remove_fft_cache=False,
        is_first_epoch=epoch == 0, hist_length=c["hist_length"], actual_step=1, fast_axis_reg_weight_positions=0,
        fast_axis_reg_weight_tilts=0, slow_axis_reg_weight_positions=0, slow_axis_reg_weight_tilts=0,
        scan_size=None, scan_step_A=1, current_deformation_reg_weight_positions=0,
        current_deformation_reg_weight_tilts=0, warnings=warnings, data_simulation_flag=False,
        data_simulation_exitwave=False, pos_puzzling=False, probe_mod_reg_weight=0, probe_mod_tol=0.05,
        use_padded_intensity=True, counter_failed_epochs=failed)


@pytest.mark.parametrize("name", LBFGS_CASES)
def test_bfgs_update_follows_reference(name):
    from pypty_gb300 import iterative
    c = load_lbfgs(name)
    ns = _fake_reference_module(c)
    fn = iterative.bind(ns)
    np.random.seed(5)
    warnings, failed = "", 0
    for e, ref in enumerate(c["ref_scalars"]):
        res = _call(fn, c, e, warnings, failed)
        total_loss, sse, _cc, step, count, dv, ndv, warnings, failed = res
        assert int(count) == int(ref[3]), (e, count, ref)
        assert float(step) == pytest.approx(float(ref[2]), rel=1e-6)
        assert float(total_loss) == pytest.approx(float(ref[0]), rel=1e-4)
        assert float(dv) == pytest.approx(float(ref[4]), rel=1e-2)
        assert failed == 0 and ns.history_bfgs["empty_hist"] is False
        assert isinstance(ns.obj, np.ndarray) and ns.obj.dtype == np.complex64
        assert rel_l2(ns.obj, c["ref_obj"][e]) <= 1e-3, (e, rel_l2(ns.obj, c["ref_obj"][e]))
        assert rel_l2(ns.probe, c["ref_probe"][e]) <= 1e-3
        if c["step_pos"]:
            assert rel_l2(ns.positions_correction, c["ref_corr"][e]) <= 1e-3


def test_bfgs_update_module_variables_and_reset():
    """This module's own variables work like the reference's; a reset empties the history."""
    from pypty_gb300 import iterative
    c = load_lbfgs("pos_lsq_sqrt")
    mod = sys.modules["pypty_gb300.iterative"]
    mod.obj, mod.probe = c["obj"].copy(), c["probe"].copy()
    mod.positions, mod.positions_correction = c["positions"].copy(), c["corr"].copy()
    mod.tilts = np.zeros((1, 6), np.float32)
    mod.tilts_correction = np.zeros((1, 6), np.float32)
    iterative.reset_bfgs_history()
    np.random.seed(5)
    r0 = _call(iterative.bfgs_update, c, 0, "", 0)
    assert int(r0[4]) == int(c["ref_scalars"][0][3])
    assert mod.history_bfgs["empty_hist"] is False
    iterative.reset_bfgs_history()
    assert mod.history_bfgs["empty_hist"] is True
    r1 = _call(iterative.bfgs_update, c, 1, "", 0)     # starts again from the first-step branch
    assert r1[5] < 0


def test_bfgs_update_refines_tilts_aberrations_and_beam_current():
    """Object, probe, per-position tilt corrections (tilt_mode 3), aberration arrays and beam
    currents refined together on the variants path: the same trial counts and steps as the
    reference's bfgs_update and the refined arrays after every call
    (tests/golden/make_golden_lbfgs.py make_refine_case)."""
    from pypty_gb300 import iterative
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "lbfgs_refine_tilts_aberr_current.npz")))
    s = d["scalars"]
    c = dict(d, distance=float(s[0]), edge_mult=float(s[1]), wavelength=float(s[2]), px=float(s[3]),
             cutoff=float(s[4]), rolloff=0.0, loss_weight=float(s[6]), batch=int(s[7]), algorithm=str(d["algorithm"]),
             step_probe=1, step_obj=1, step_pos=0, orthogonal=False, lazy_clean=False, hist_length=10)
    ns = types.SimpleNamespace(obj=c["obj"].copy(), probe=c["probe"].copy(), positions=c["positions"].copy(),
                               positions_correction=c["pos_correction"].astype(np.float32).copy(),
                               tilts=c["tilts"].copy(), tilts_correction=np.zeros_like(c["tilts"]),
                               static_background=None, aberrations_array=c["aberrations"].copy(),
                               beam_current=c["beam_current"].copy(), history_bfgs=None)
    fn = iterative.bind(ns)
    np.random.seed(5)
    warnings, failed = "", 0
    f = np.float32
    step = 1e-3    # the generator's float first step, then the accepted one
    for e, ref in enumerate(c["ref_scalars"]):
        kw = dict(this_step_tilts=1, tilt_mode=3, aberration_marker=c["aberration_marker"],
                  this_step_aberrations_array=1, this_beam_current_step=1, actual_step=step)
        res = _call_with(fn, c, e, warnings, failed, kw)
        total_loss, sse, _cc, step, count, dv, ndv, warnings, failed = res
        print(e, count, step, total_loss, "ref", ref[3], ref[2], ref[0])
        assert int(count) == int(ref[3]), (e, count, ref)
        assert float(step) == pytest.approx(float(ref[2]), rel=1e-5)
        assert float(total_loss) == pytest.approx(float(ref[0]), rel=1e-4)
        assert failed == 0
        assert rel_l2(ns.obj, c["ref_obj"][e]) <= 1e-3
        assert rel_l2(ns.probe, c["ref_probe"][e]) <= 1e-3
        assert rel_l2(ns.tilts_correction, c["ref_tcorr"][e]) <= 2e-3, (e, rel_l2(ns.tilts_correction,
                                                                              c["ref_tcorr"][e]))
        assert rel_l2(ns.aberrations_array, c["ref_ab"][e]) <= 1e-3
        assert rel_l2(ns.beam_current, c["ref_bc"][e]) <= 1e-3
        assert isinstance(ns.tilts_correction, np.ndarray) and ns.tilts_correction.dtype == f


def test_bfgs_update_refines_the_static_background():
    """Object, probe and static background refined together (the reference's
    update_static_background): the same trial counts and steps as the reference's bfgs_update
    and the background after every call (tests/golden/make_golden_lbfgs.py make_static_case)."""
    from pypty_gb300 import iterative
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "lbfgs_refine_static_background.npz")))
    s = d["scalars"]
    c = dict(d, distance=float(s[0]), edge_mult=float(s[1]), wavelength=float(s[2]), px=float(s[3]),
             cutoff=float(s[4]), rolloff=0.0, loss_weight=float(s[6]), batch=int(s[7]), algorithm=str(d["algorithm"]),
             step_probe=1, step_obj=1, step_pos=0, orthogonal=False, lazy_clean=False, hist_length=10)
    ns = types.SimpleNamespace(obj=c["obj"].copy(), probe=c["probe"].copy(), positions=c["positions"].copy(),
                               positions_correction=c["pos_correction"].astype(np.float32).copy(),
                               tilts=np.zeros((1, 6), np.float32), tilts_correction=np.zeros((1, 6), np.float32),
                               static_background=c["static_background"].copy(), aberrations_array=None,
                               beam_current=None, history_bfgs=None)
    fn = iterative.bind(ns)
    np.random.seed(6)
    warnings, failed = "", 0
    step = 1.0
    for e, ref in enumerate(c["ref_scalars"]):
        res = _call_with(fn, c, e, warnings, failed, dict(this_step_static_background=1, actual_step=step))
        total_loss, sse, _cc, step, count, dv, ndv, warnings, failed = res
        print(e, count, step, total_loss, "ref", ref[3], ref[2], ref[0])
        assert int(count) == int(ref[3]), (e, count, ref)
        assert float(step) == pytest.approx(float(ref[2]), rel=1e-5)
        assert float(total_loss) == pytest.approx(float(ref[0]), rel=1e-4)
        assert failed == 0
        assert rel_l2(ns.obj, c["ref_obj"][e]) <= 1e-3
        assert rel_l2(ns.probe, c["ref_probe"][e]) <= 1e-3
        assert rel_l2(ns.static_background, c["ref_sb"][e]) <= 1e-3
        assert isinstance(ns.static_background, np.ndarray) and ns.static_background.dtype == np.float32


def test_bfgs_update_with_probe_scenarios():
    """Two probe scenarios (a 4D probe with probe_marker) whose modes are kept orthogonal:
    the same trial counts and steps as the reference's bfgs_update, object and 4D probe after
    every call (tests/golden/make_golden_lbfgs.py make_scenario_case)."""
    from pypty_gb300 import iterative
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "lbfgs_refine_probe_scenarios.npz")))
    s = d["scalars"]
    c = dict(d, distance=float(s[0]), edge_mult=float(s[1]), wavelength=float(s[2]), px=float(s[3]),
             cutoff=float(s[4]), rolloff=0.0, loss_weight=float(s[6]), batch=int(s[7]), algorithm=str(d["algorithm"]),
             step_probe=1, step_obj=1, step_pos=0, orthogonal=True, lazy_clean=False, hist_length=10)
    ns = types.SimpleNamespace(obj=c["obj"].copy(), probe=c["probe"].copy(), positions=c["positions"].copy(),
                               positions_correction=c["pos_correction"].astype(np.float32).copy(),
                               tilts=np.zeros((1, 6), np.float32), tilts_correction=np.zeros((1, 6), np.float32),
                               static_background=None, aberrations_array=None, beam_current=None, history_bfgs=None)
    fn = iterative.bind(ns)
    np.random.seed(7)
    warnings, failed = "", 0
    step = 1.0
    for e, ref in enumerate(c["ref_scalars"]):
        res = _call_with(fn, c, e, warnings, failed, dict(probe_marker=c["probe_marker"], actual_step=step))
        total_loss, sse, _cc, step, count, dv, ndv, warnings, failed = res
        print(e, count, step, total_loss, "ref", ref[3], ref[2], ref[0])
        assert int(count) == int(ref[3]), (e, count, ref)
        assert float(step) == pytest.approx(float(ref[2]), rel=1e-5)
        assert float(total_loss) == pytest.approx(float(ref[0]), rel=1e-4)
        assert rel_l2(ns.obj, c["ref_obj"][e]) <= 1e-3
        assert ns.probe.shape == c["probe"].shape
        assert rel_l2(ns.probe, c["ref_probe"][e]) <= 1e-3


def _call_with(fn, c, epoch, warnings, failed, over):
    """_call with some arguments replaced (the refinement flags of the variants path)."""
    captured = {}

    def grab(**kw):
        captured.update(kw)
        return None
    _call(grab, c, epoch, warnings, failed)
    captured.update(over)
    return fn(**captured)
