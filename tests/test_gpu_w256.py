"""256-px windows (clusters of four blocks, modes processed in turn): FFT against NumPy,
the loss-and-gradient path and its forward/adjoint split against the FP64 oracle."""
import numpy as np
import pytest

from golden_io import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("inverse,shift", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_window_fft_256_matches_numpy(inverse, shift):
    import torch
    from pypty_gb300.engine import Engine
    eng = Engine(torch.device("cuda", 0))
    rng = np.random.default_rng(11 + 2 * inverse + shift)
    x = (rng.normal(size=(3, 256, 256)) + 1j * rng.normal(size=(3, 256, 256))).astype(np.complex64)
    out = eng.fft2(torch.from_numpy(x).cuda(), inverse=bool(inverse), shift=bool(shift)).cpu().numpy()
    xd = x.astype(np.complex128)
    if not inverse:
        ref = np.fft.fft2(xd, axes=(1, 2))
        ref = np.fft.fftshift(ref, axes=(1, 2)) if shift else ref
    else:
        ref = np.fft.ifft2(np.fft.ifftshift(xd, axes=(1, 2)) if shift else xd, axes=(1, 2))
    assert rel_l2(out, ref) <= 2e-6


def _case(Z, Mp, Mo, alg, seed, n_scan=2, rolloff=0.0, edge=1.0, distances=None):
    from oracle import ptycho_oracle as orc
    from pypty_gb300 import synth
    rng = np.random.default_rng(seed)
    px, kV, W = 0.1, 300.0, 256
    n = W + n_scan * 9 + 8
    truth = synth.gaussian_phase_object(n, n, Z, 120, 0.3, px, 0.2, 1.0, rng, n_modes=Mo)
    probe = synth.make_probe(W, px, kV, 30.0, 60.0, Mp, 0.5 ** np.arange(Mp), 1e5)
    ipos, corr = synth.split_positions(synth.raster_positions(n_scan, n_scan, 9.0, 2.0, rng))
    lam = synth.wavelength_A(kV)
    seq = np.arange(ipos.shape[0])
    dist = 1.0 if distances is None else np.asarray(distances, np.float32)
    sim = orc.loss_and_direction(truth, probe, ipos, corr, dist, edge, None, alg, lam, 1, 1, 1, px, px, 2 / 3,
                                 rolloff, seq, 1, 4, simulate=True)
    meas = synth.poisson_patterns(sim, 1.0, rng)
    obj0 = np.exp(0.6j * np.angle(truth)).astype(np.complex64)
    c = dict(obj=obj0, probe=probe, positions=ipos, pos_correction=corr, sequence=seq, measured=meas,
             algorithm=alg, wavelength=lam, px=px, cutoff=2 / 3, rolloff=rolloff, distance=1.0, edge_mult=edge,
             loss_weight=1, batch=3, step_obj=1, step_probe=1, step_pos=1, distances=distances)
    ref = orc.loss_and_direction(obj0.astype(np.complex128), probe.astype(np.complex128), ipos,
                                 corr.astype(np.float64), dist, edge, meas.astype(np.float64), alg, lam, 1, 1, 1, px,
                                 px, 2 / 3, rolloff, seq, 1, 3, float_dtype=np.float64, complex_dtype=np.complex128)
    return c, ref


@pytest.mark.parametrize("Z,Mp,Mo,alg,rolloff,edge", [(3, 2, 1, "lsq_sqrt", 0.0, 1.0), (2, 3, 2, "lsq", 0.1, 1.0),
                                                     (3, 5, 1, "ml", 0.0, 1.5)])
def test_w256_against_fp64_oracle(Z, Mp, Mo, alg, rolloff, edge):
    from gpu_helpers import run_gpu
    c, ref = _case(Z, Mp, Mo, alg, seed=Z * 10 + Mp, rolloff=rolloff, edge=edge)
    loss, sse, og, pg, posg = run_gpu(c)
    assert abs(loss - ref[0]) <= 1e-5 * abs(ref[0])
    assert rel_l2(og, ref[2]) <= 1e-4
    assert rel_l2(pg, ref[3]) <= 1e-4
    assert rel_l2(posg, ref[4]) <= 1e-4


@pytest.mark.parametrize("ckpt", [1, 2])
def test_w256_per_slice_distances_against_fp64_oracle(ckpt):
    """One distance per slice step (the reference's this_distances with Z - 1 entries), with a
    thick first slice, kept or recomputed in the adjoint."""
    c, ref = _case(4, 2, 1, "lsq_sqrt", seed=77, edge=1.4, distances=[0.8, 1.6, 2.4])
    ls, og, pg, posg = _run_with(c, checkpoint_every=ckpt, slice_distances=c["distances"])
    loss = float(ls[0])
    assert abs(loss - ref[0]) <= 1e-5 * abs(ref[0])
    assert rel_l2(og, ref[2]) <= 1e-4
    assert rel_l2(pg, ref[3]) <= 1e-4
    assert rel_l2(posg, ref[4]) <= 1e-4


def test_w256_forward_adjoint_split_matches_one_shot():
    import torch
    from gpu_helpers import run_gpu
    from pypty_gb300.engine import Engine, Geometry, make_problem
    c, _ = _case(2, 2, 1, "lsq_sqrt", seed=3)
    one = run_gpu(c)
    dev = torch.device("cuda", 0)
    eng = Engine(dev)
    geo = Geometry.make(c["positions"], c["pos_correction"], c["sequence"])
    prob = make_problem(256, c["obj"].shape, 2, geo, algorithm="lsq_sqrt", wavelength=c["wavelength"],
                        pixel_size_x=c["px"], pixel_size_y=c["px"], slice_distance=1.0, step_pos=True)
    ls, ws = eng.forward(prob, torch.from_numpy(c["obj"]).to(dev), torch.from_numpy(c["probe"]).to(dev), geo,
                         torch.from_numpy(c["measured"]).to(dev))
    _, og, pg, posg = eng.backward(prob, ws)
    torch.cuda.synchronize()
    assert abs(ls[0].item() - one[0]) <= 1e-9 * abs(one[0])
    assert rel_l2(og.cpu().numpy(), one[2]) <= 1e-6
    assert rel_l2(pg.cpu().numpy(), one[3]) <= 1e-6
    assert rel_l2(posg.cpu().numpy(), one[4]) <= 1e-6


def _run_with(c, **kw):
    import torch
    from pypty_gb300.engine import Engine, Geometry, make_problem
    dev = torch.device("cuda", 0)
    eng = Engine(dev)
    geo = Geometry.make(c["positions"], c["pos_correction"], c["sequence"])
    W = c["probe"].shape[0]
    prob = make_problem(W, c["obj"].shape, c["probe"].shape[2], geo, algorithm=c["algorithm"],
                        wavelength=c["wavelength"], pixel_size_x=c["px"], pixel_size_y=c["px"],
                        slice_distance=c["distance"], edge_mult=c["edge_mult"], smooth_rolloff=c["rolloff"],
                        compute_batch=c["batch"], step_pos=True, **kw)
    out = eng.loss_and_direction(prob, torch.from_numpy(np.ascontiguousarray(c["obj"])).to(dev),
                                 torch.from_numpy(np.ascontiguousarray(c["probe"])).to(dev), geo,
                                 torch.from_numpy(np.ascontiguousarray(c["measured"])).to(dev))
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in out]


@pytest.mark.parametrize("ckpt", [2, 3, 5])
def test_recomputation_checkpointing_gives_identical_gradients(ckpt):
    """Keeping every k-th slice and recomputing the rest reproduces the gradients bit for bit."""
    c, _ = _case(5, 2, 1, "lsq_sqrt", seed=21, edge=1.5)
    full = _run_with(c, checkpoint_every=1)
    part = _run_with(c, checkpoint_every=ckpt)
    for x, y in zip(full, part):
        assert np.array_equal(x, y)


def test_checkpointed_gradient_matches_finite_differences():
    """Large-adjoint style check: phases of 64 random object pixels and the probe-mode
    amplitudes, central differences of the loss against the checkpointed gradient."""
    import torch
    from pypty_gb300.autograd import multislice_loss
    c, _ = _case(6, 3, 1, "lsq_sqrt", seed=33)
    dev = torch.device("cuda", 0)
    obj = torch.from_numpy(c["obj"]).to(dev)
    probe = torch.from_numpy(c["probe"]).to(dev)
    corr = torch.from_numpy(c["pos_correction"])
    meas = torch.from_numpy(c["measured"]).to(dev)
    kw = dict(algorithm="lsq_sqrt", wavelength=c["wavelength"], pixel_size_x=c["px"], pixel_size_y=c["px"],
              slice_distance=c["distance"])
    # gradient with checkpointing (every 3rd slice kept)
    res = _run_with(c, checkpoint_every=3)
    loss0, g_obj, g_probe = float(res[0][0]), res[1], res[2]
    z0 = c["obj"].astype(np.complex128)
    # dL/dphi per pixel: 2 Re(conj(dL/dz*) * i z); perturb the phases of the 64 pixels with the
    # largest |dL/dphi| (sign along it), so the loss change stands well above float32 noise
    dldphi = 2 * np.real(np.conj(g_obj.astype(np.complex128)) * 1j * z0)
    top = np.argsort(np.abs(dldphi).ravel())[-64:]
    dphi = np.zeros(z0.size, np.float64)
    dphi[top] = np.sign(dldphi.ravel()[top])
    dphi = dphi.reshape(z0.shape)
    slope = float(np.sum(dldphi * dphi))

    def L(o, p):
        with torch.no_grad():
            return multislice_loss(torch.from_numpy(o.astype(np.complex64)).to(dev),
                                   torch.from_numpy(p.astype(np.complex64)).to(dev), corr, c["positions"], meas,
                                   **kw).item()
    h = 5e-3
    fd = (L(z0 * np.exp(1j * h * dphi), c["probe"]) - L(z0 * np.exp(-1j * h * dphi), c["probe"])) / (2 * h)
    assert abs(fd - slope) <= 2e-2 * abs(slope) + 1e-6 * abs(loss0), (fd, slope)
    # probe-mode amplitude coefficients: P_j -> (1 + t) P_j
    p0 = c["probe"].astype(np.complex128)
    for j in range(p0.shape[2]):
        dp = np.zeros_like(p0)
        dp[:, :, j] = p0[:, :, j]
        slope = float(np.sum(2 * np.real(np.conj(g_probe.astype(np.complex128)) * dp)))
        hp = 1e-3
        fd = (L(c["obj"], p0 + hp * dp) - L(c["obj"], p0 - hp * dp)) / (2 * hp)
        assert abs(fd - slope) <= 2e-2 * abs(slope) + 1e-6 * abs(loss0), (j, fd, slope)
