"""Install the GPU path into an imported reference ``pypty`` package.

The reference calls its hot path through module attributes
(``pyptyobjective.loss_and_direction`` at ``pypty/iterative.py:524,773``), so replacing the
attribute is enough for ``pypty.iterative.run`` to use the GB300 kernels.
"""
from __future__ import annotations

from . import objective as _objective

_SAVED = {}


def install(pypty_module, multislice_core: bool = False, iterative: bool = False) -> None:
    """Point ``pypty.objective.loss_and_direction`` at the GPU implementation; with
    ``multislice_core=True`` also ``pypty.multislice_core.multislice`` /
    ``multislice_grads`` / ``scatteradd`` (used by reference code that calls them
    directly; ``loss_and_direction`` on the GPU path does not go through them). With
    ``iterative=True`` also ``pypty.iterative.bfgs_update`` (bound to the module variables
    of ``pypty.iterative``, ``pypty/iterative.py:419,440``) and ``pypty.utils.fourier_clean``:
    the whole optimizer step of ``pypty.iterative.run`` then runs on the device."""
    obj_mod = pypty_module.objective
    if iterative:
        from . import iterative as _it
        from . import utils as _ut
        it_mod = pypty_module.iterative
        if "iterative.bfgs_update" not in _SAVED:
            _SAVED["iterative.bfgs_update"] = (it_mod, it_mod.bfgs_update)
        it_mod.bfgs_update = _it.bind(it_mod)
        ut_mod = pypty_module.utils
        if "utils.fourier_clean" not in _SAVED:
            _SAVED["utils.fourier_clean"] = (ut_mod, ut_mod.fourier_clean)
        ut_mod.fourier_clean = _ut.fourier_clean
    if "loss_and_direction" not in _SAVED:
        _SAVED["loss_and_direction"] = (obj_mod, obj_mod.loss_and_direction)
    obj_mod.loss_and_direction = _objective.loss_and_direction
    if multislice_core:
        from . import multislice_core as _mc
        ms_mod = pypty_module.multislice_core
        for name in ("multislice", "multislice_grads", "scatteradd"):
            key = "multislice_core." + name
            if key not in _SAVED:
                _SAVED[key] = (ms_mod, getattr(ms_mod, name))
            setattr(ms_mod, name, getattr(_mc, name))


def uninstall() -> None:
    """Restore the attributes replaced by ``install``."""
    for key, (mod, fn) in list(_SAVED.items()):
        setattr(mod, key.split(".")[-1], fn)
        del _SAVED[key]
