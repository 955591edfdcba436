"""The launch-graph cache of pty_loss_and_direction: the second call with the same problem and
buffers captures the launch sequence, later calls replay it. Replays must see the caller's
current buffer contents (object values, host geometry) and give exactly the results of a
direct launch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(W=64, Z=3, Mp=2, n_scan=4, seed=3):
    from pypty_gb300 import synth
    rng = np.random.default_rng(seed)
    px, kV = 0.15, 300.0
    n = W + 8 * n_scan + 8
    truth = synth.gaussian_phase_object(n, n, Z, 40, 0.3, px, 0.2, 0.9, rng)
    probe = synth.make_probe(W, px, kV, 30.0, 40.0, Mp, [0.7, 0.3][:Mp], 1e4)
    ipos, corr = synth.split_positions(synth.raster_positions(n_scan, n_scan, 8.0, 1.5, rng))
    meas = rng.poisson(20.0, (ipos.shape[0], W, W)).astype(np.float32)
    return truth, probe, ipos, corr, meas, synth.wavelength_A(kV), px


@pytest.mark.parametrize("batch", [16, 5])
def test_graph_replays_match_direct_launches(batch):
    import torch
    from pypty_gb300.engine import Engine, Geometry, make_problem
    truth, probe, ipos, corr, meas, lam, px = _case()
    dev = torch.device("cuda", 0)
    cached = Engine(dev)
    obj_d = torch.from_numpy(np.exp(0.5j * np.angle(truth)).astype(np.complex64)).to(dev)
    probe_d = torch.from_numpy(probe).to(dev)
    meas_d = torch.from_numpy(meas).to(dev)
    out = (torch.empty(2, dtype=torch.float64, device=dev), torch.empty_like(obj_d), torch.empty_like(probe_d),
           torch.empty((ipos.shape[0], 2), dtype=torch.float32, device=dev))
    rng = np.random.default_rng(11)
    keep = []   # the direct launches' engines and buffers stay alive: no address is reused
    for call in range(5):
        # new object values in the same buffer and new sub-pixel corrections every call
        obj_d.copy_(torch.from_numpy(np.exp((0.4 + 0.05 * call) * 1j * np.angle(truth)).astype(np.complex64)))
        c = (corr + rng.uniform(-0.1, 0.1, corr.shape)).astype(np.float32)
        geo = Geometry.make(ipos, c)
        prob = make_problem(64, truth.shape, probe.shape[2], geo, algorithm="ml", wavelength=lam, pixel_size_x=px,
                            pixel_size_y=px, slice_distance=2.0, compute_batch=batch, step_pos=True)
        got = cached.loss_and_direction(prob, obj_d, probe_d, geo, meas_d, out=out)
        got = [t.cpu().numpy().copy() for t in got]
        direct = (Engine(dev), obj_d.clone(), probe_d.clone(), meas_d.clone())
        keep.append(direct)
        ref = direct[0].loss_and_direction(prob, direct[1], direct[2], geo, direct[3])
        keep.append(ref)
        ref = [t.cpu().numpy() for t in ref]
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), "call %d differs from a direct launch" % call
    assert graph_cache_info()["graphs"] >= 2     # the two staging buffers' keys were captured
    assert graph_cache_info()["replays"] >= 1


def graph_cache_info():
    import ctypes
    from pypty_gb300 import _lib
    k, g, u = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    r = ctypes.c_int64()
    _lib.check(_lib.lib().pty_graph_cache_info(ctypes.byref(k), ctypes.byref(g), ctypes.byref(u), ctypes.byref(r)),
               "pty_graph_cache_info")
    return dict(keys=k.value, graphs=g.value, uncapturable=u.value, replays=r.value)
