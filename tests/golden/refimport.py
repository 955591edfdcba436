"""Import the reference pypty package on a machine without h5py/matplotlib/skimage/CuPy.

Used only by ``make_golden.py`` (fixture generation, run where the reference sources are
mounted). The reference imports those packages at module level but the NumPy
loss-and-gradient path never calls them, so empty stand-in modules are enough. Without
CuPy the reference falls back to NumPy/SciPy (``pypty/fft.py:4-6``,
``pypty/objective.py:7-37``).
"""
import os
import sys
import types

# the checkout of the reference sources; required (no default location)
REFERENCE_ROOT = os.environ.get("PYPTY_REFERENCE_ROOT", "")


class _Anything:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()


def _stub(name, **attrs):
    mod = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def import_reference():
    """Return the reference ``pypty`` package (NumPy backend)."""
    if "pypty" in sys.modules and hasattr(sys.modules["pypty"], "objective"):
        return sys.modules["pypty"]
    if not REFERENCE_ROOT or not os.path.isdir(os.path.join(REFERENCE_ROOT, "pypty")):
        raise ImportError("set PYPTY_REFERENCE_ROOT to the reference checkout (the directory holding pypty/); "
                          "got %r" % REFERENCE_ROOT)
    _stub("h5py", File=_Anything)
    mpl = _stub("matplotlib")
    for sub in ["pyplot", "patches", "patheffects", "colors", "cm", "gridspec"]:
        setattr(mpl, sub, _stub("matplotlib." + sub))
    sys.modules["matplotlib.patches"].Circle = _Anything
    sys.modules["matplotlib.patches"].Rectangle = _Anything
    sk = _stub("skimage")
    for sub in ["filters", "measure", "morphology", "restoration", "transform", "feature",
                "registration"]:
        setattr(sk, sub, _stub("skimage." + sub))
    sys.path.insert(0, REFERENCE_ROOT)
    import pypty  # noqa: F401
    from pypty import objective, multislice_core, fft, utils  # noqa: F401
    return sys.modules["pypty"]
