"""Pin the optimizer oracle (``fourier_clean``, ``bfgs_update``) to the reference's outputs."""
import numpy as np
import pytest

from golden_io import rel_l2
from oracle import lbfgs_oracle as lo

LBFGS_CASES = ["obj_probe_ml", "pos_lsq_sqrt", "rolloff_orth_lazy"]


def load_lbfgs(name):
    d = dict(np.load("tests/golden/lbfgs_%s.npz" % name))
    s = d["scalars"]
    o = d["opts"]
    c = dict(obj=d["obj"], probe=d["probe"], positions=d["positions"], corr=d["pos_correction"].astype(np.float32),
             measured=d["measured"], sequence=d["sequence"], distance=float(s[0]), edge_mult=float(s[1]),
             wavelength=float(s[2]), px=float(s[3]), cutoff=float(s[4]), loss_weight=float(s[6]),
             batch=int(s[7]), algorithm=str(d["algorithm"]), step_obj=bool(o[0]), step_probe=bool(o[1]),
             step_pos=bool(o[2]), rolloff=float(o[3]), orthogonal=bool(o[4]), lazy_clean=bool(o[6]),
             hist_length=int(o[7]), ref_scalars=d["ref_scalars"], ref_obj=d["ref_obj"], ref_probe=d["ref_probe"],
             ref_corr=d["ref_corr"])
    return c


def oracle_problem(c):
    return lo.Problem(c["positions"], c["distance"], c["edge_mult"], c["measured"], c["algorithm"],
                      c["wavelength"], c["px"], c["px"], c["cutoff"], c["sequence"], c["loss_weight"], c["batch"])


def run_oracle_epochs(c):
    opt = lo.BfgsOracle(oracle_problem(c), c["obj"], c["probe"], c["corr"])
    np.random.seed(5)
    out = []
    for _ in range(len(c["ref_scalars"])):
        r = opt.update(step_obj=c["step_obj"], step_probe=c["step_probe"], step_pos=c["step_pos"],
                       cutoff=np.float32(c["cutoff"]), rolloff=np.float32(c["rolloff"]), lazy_clean=c["lazy_clean"],
                       orthogonal=c["orthogonal"], c1=0.1, c2=0.9, max_count=20, hist_length=c["hist_length"])
        out.append((r, opt.obj.copy(), opt.probe.copy(), opt.corr.copy()))
    return out


def test_fourier_clean_oracle_matches_reference():
    d = dict(np.load("tests/golden/fourier_clean_c64.npz"))
    for name in ["a2", "a3", "a4", "a4r"]:
        cut, roll = d[name + "_cut"]
        res = lo.fourier_clean(d[name + "_in"], cutoff=np.float32(cut), rolloff=np.float32(roll))
        assert rel_l2(res, d[name + "_out"]) <= 1e-6, name
    res = lo.fourier_clean(d["m_in"], mask=d["m_mask"])
    assert rel_l2(res, d["m_out"]) <= 1e-6


@pytest.mark.parametrize("name", LBFGS_CASES)
def test_bfgs_oracle_matches_reference(name):
    c = load_lbfgs(name)
    out = run_oracle_epochs(c)
    for e, ((loss, sse, step, count, dv, ndv, accepted), obj, probe, corr) in enumerate(out):
        ref = c["ref_scalars"][e]
        assert accepted
        assert int(count) == int(ref[3]), (e, count, ref[3])
        assert float(step) == pytest.approx(float(ref[2]), rel=1e-6)
        assert float(loss) == pytest.approx(float(ref[0]), rel=1e-5)
        assert float(dv) == pytest.approx(float(ref[4]), rel=1e-3)
        assert rel_l2(obj, c["ref_obj"][e]) <= 1e-4, (e, rel_l2(obj, c["ref_obj"][e]))
        assert rel_l2(probe, c["ref_probe"][e]) <= 1e-4
        if c["step_pos"]:
            assert rel_l2(corr, c["ref_corr"][e]) <= 1e-4


def test_orthogonalise_modes():
    rng = np.random.default_rng(0)
    p = (rng.normal(size=(32, 32, 3)) + 1j * rng.normal(size=(32, 32, 3))).astype(np.complex64)
    q = lo.make_states_orthogonal(p).astype(np.complex128)
    for i in range(3):
        for j in range(i):
            ov = np.sum(np.conjugate(q[:, :, j]) * q[:, :, i])
            assert abs(ov) <= 1e-4 * np.sqrt(np.sum(np.abs(q[:, :, i]) ** 2) * np.sum(np.abs(q[:, :, j]) ** 2))
