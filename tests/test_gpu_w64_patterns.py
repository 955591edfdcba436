"""The 64-px fused kernel copies each position's measured pattern into shared memory at the start
of its block: 16-byte asynchronous copies when the pattern starts on a 16-byte boundary, 4-byte
copies otherwise. A pattern array that starts 4 bytes into its buffer takes the second route and
must give exactly the result of the aligned array (same values, same arithmetic)."""
import numpy as np
import pytest

from golden_io import load_case
from gpu_helpers import run_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["single_slice_c64", "multislice_ml_c64"])
def test_unaligned_patterns_match_aligned(name):
    import torch
    c = load_case(name)
    assert np.asarray(c["probe"]).shape[0] == 64
    meas = np.ascontiguousarray(c["measured"]).astype(np.float32)
    dev = torch.device("cuda", 0)
    aligned = run_gpu(c)
    buf = torch.zeros(meas.size + 1, dtype=torch.float32, device=dev)
    buf[1:].copy_(torch.from_numpy(meas.ravel()).to(dev))
    shifted = buf[1:].view(meas.shape)
    assert shifted.data_ptr() % 16 != 0
    got = run_gpu(c, measured=shifted)
    torch.cuda.synchronize()
    assert got[0] == aligned[0] and got[1] == aligned[1]
    for a, b in zip(aligned[2:], got[2:]):
        assert np.array_equal(a, b)
