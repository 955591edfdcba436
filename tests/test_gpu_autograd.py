"""The autograd function: gradients against the reference (golden), the one-shot call, and
central finite differences of the loss."""
import numpy as np
import pytest

from golden_io import load_case, rel_l2

pytestmark = pytest.mark.gpu


def _tensors(c):
    import torch
    dev = torch.device("cuda", 0)
    obj = torch.from_numpy(np.ascontiguousarray(c["obj"]).astype(np.complex64)).to(dev)
    probe = torch.from_numpy(np.ascontiguousarray(c["probe"]).astype(np.complex64)).to(dev)
    corr = torch.from_numpy(np.ascontiguousarray(c["pos_correction"]).astype(np.float32))
    meas = torch.from_numpy(np.ascontiguousarray(c["measured"]).astype(np.float32)).to(dev)
    return obj, probe, corr, meas


def _loss(c, obj, probe, corr, meas):
    from pypty_gb300.autograd import multislice_loss
    return multislice_loss(obj, probe, corr, c["positions"], meas, algorithm=c["algorithm"],
                           wavelength=float(np.float32(c["wavelength"])), pixel_size_x=float(np.float32(c["px"])),
                           pixel_size_y=float(np.float32(c["px"])), slice_distance=c["distance"],
                           sequence=c["sequence"], edge_mult=c["edge_mult"],
                           damping_cutoff=float(np.float32(c["cutoff"])),
                           smooth_rolloff=float(np.float32(c["rolloff"])), loss_weight=c["loss_weight"],
                           probe_shift=bool(np.any(c["pos_correction"] != 0)) or bool(c["step_pos"]))


@pytest.mark.parametrize("name", ["multislice_ml_c64", "modes_lsq_c64", "w128_modes_c64"])
def test_autograd_matches_reference_gradient(name):
    c = load_case(name)
    obj, probe, corr, meas = _tensors(c)
    obj.requires_grad_(True)
    probe.requires_grad_(True)
    corr.requires_grad_(bool(c["step_pos"]))
    loss = _loss(c, obj, probe, corr, meas)
    loss.backward()
    assert abs(loss.item() - float(c["ref_loss"])) <= 1e-5 * abs(float(c["ref_loss"]))
    # torch's gradient of a real loss is 2 dL/dz*; the reference returns dL/dz*
    assert rel_l2(obj.grad.cpu().numpy() / 2, c["ref_object_grad"]) <= 1e-4
    assert rel_l2(probe.grad.cpu().numpy() / 2, np.asarray(c["ref_probe_grad"]).reshape(probe.shape)) <= 1e-4
    if c["step_pos"]:
        assert rel_l2(corr.grad.numpy(), c["ref_pos_grad"]) <= 1e-4


def test_loss_without_grad_skips_adjoint():
    c = load_case("multislice_ml_c64")
    obj, probe, corr, meas = _tensors(c)
    loss = _loss(c, obj, probe, corr, meas)
    assert not loss.requires_grad
    assert abs(loss.item() - float(c["ref_loss"])) <= 1e-5 * abs(float(c["ref_loss"]))


@pytest.mark.parametrize("name,what,alg", [("multislice_ml_c64", "obj", "lsq_sqrt"),
                                           ("multislice_ml_c64", "probe", "lsq"),
                                           ("w128_modes_c64", "obj", None), ("modes_lsq_c64", "probe", None),
                                           ("single_slice_c64", "pos", None)])
def test_gradient_matches_central_finite_differences(name, what, alg):
    """dL along a random direction d: (L(x + h d) - L(x - h d)) / 2h = Re<grad, d>.

    The Poisson loss ("ml") is too curved at these evaluation points for a central
    difference of float32 evaluations (its FP64 difference needs steps of 1e-7 relative);
    its gradient is checked against the reference's own gradient instead, and the
    multislice inputs of that case are differentiated here with the amplitude and
    intensity losses."""
    import torch
    c = load_case(name)
    if alg is not None:
        c = dict(c, algorithm=alg)
    obj, probe, corr, meas = _tensors(c)
    x = {"obj": obj, "probe": probe, "pos": corr}[what]
    x.requires_grad_(True)
    loss = _loss(c, obj, probe, corr, meas)
    loss.backward()
    g = x.grad.detach().clone()
    rng = np.random.default_rng(5)
    if x.is_complex():
        d = torch.from_numpy((rng.normal(size=x.shape) + 1j * rng.normal(size=x.shape)).astype(np.complex64))
    else:
        d = torch.from_numpy(rng.normal(size=x.shape).astype(np.float32))
    d = (d / torch.linalg.vector_norm(d)).to(x.device)
    slope = float(torch.real(torch.vdot(g.reshape(-1).to(torch.complex128), d.reshape(-1).to(torch.complex128))))
    # step: a relative change of the loss of about 1e-5 -- small enough for the central
    # difference's truncation error (FP64 oracle: ~1e-4 on these cases), large enough for
    # float32 evaluation noise
    h = 1e-5 * abs(loss.item()) / max(abs(slope), 1e-30)
    h = min(h, 1e-2 * float(torch.linalg.vector_norm(x.detach().to(torch.complex128))))
    with torch.no_grad():
        vals = []
        for sgn in (1.0, -1.0):
            xs = (x.detach() + sgn * h * d).contiguous()
            args = {"obj": obj.detach(), "probe": probe.detach(), "pos": corr.detach()}
            args[what] = xs if what != "pos" else xs.cpu()
            vals.append(_loss(c, args["obj"], args["probe"], args["pos"], meas).item())
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(fd - slope) <= 5e-3 * abs(slope), (fd, slope)
