"""Install the GPU path into an imported reference ``pypty`` package.

The reference calls its hot path through module attributes
(``pyptyobjective.loss_and_direction`` at ``pypty/iterative.py:524,773``), so replacing the
attribute is enough for ``pypty.iterative.run`` to use the GB300 kernels.
"""
from __future__ import annotations

from . import objective as _objective

_SAVED = {}


def install(pypty_module) -> None:
    """Point ``pypty.objective.loss_and_direction`` at the GPU implementation."""
    obj_mod = pypty_module.objective
    if "loss_and_direction" not in _SAVED:
        _SAVED["loss_and_direction"] = (obj_mod, obj_mod.loss_and_direction)
    obj_mod.loss_and_direction = _objective.loss_and_direction


def uninstall() -> None:
    """Restore the attributes replaced by ``install``."""
    for name, (mod, fn) in list(_SAVED.items()):
        setattr(mod, name, fn)
        del _SAVED[name]
