"""Run the GPU path on a golden/oracle case (used by the gpu-marked tests)."""
import numpy as np


def run_gpu(c, compute_batch=None, engine=None, measured=None):
    """measured: a device tensor to pass instead of the case's patterns (same values)."""
    import torch
    from pypty_gb300.engine import Engine, Geometry, make_problem
    dev = torch.device("cuda", 0)
    eng = engine or Engine(dev)
    obj = np.ascontiguousarray(c["obj"]).astype(np.complex64)
    probe = np.ascontiguousarray(c["probe"]).astype(np.complex64)
    geo = Geometry.make(c["positions"], c["pos_correction"], c["sequence"])
    W = probe.shape[0]
    prob = make_problem(W, obj.shape, probe.shape[2], geo, algorithm=c["algorithm"],
                        wavelength=float(np.float32(c["wavelength"])), pixel_size_x=float(np.float32(c["px"])),
                        pixel_size_y=float(np.float32(c["px"])), slice_distance=c["distance"],
                        edge_mult=c["edge_mult"], damping_cutoff=float(np.float32(c["cutoff"])),
                        smooth_rolloff=float(np.float32(c["rolloff"])), loss_weight=c["loss_weight"],
                        compute_batch=compute_batch or c["batch"], step_obj=c["step_obj"],
                        step_probe=c["step_probe"], step_pos=c["step_pos"], slice_distances=c.get("distances"))
    if measured is None:
        measured = torch.from_numpy(np.ascontiguousarray(c["measured"]).astype(np.float32)).to(dev)
    ls, og, pg, posg = eng.loss_and_direction(
        prob, torch.from_numpy(obj).to(dev), torch.from_numpy(probe).to(dev), geo, measured)
    torch.cuda.synchronize()
    ls = ls.cpu().numpy()
    return float(ls[0]), float(ls[1]), og.cpu().numpy(), pg.cpu().numpy(), posg.cpu().numpy()
